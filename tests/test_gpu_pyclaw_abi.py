"""The PyClaw C interface on the GPU, driven through ctypes like PeanoClaw's
Python package drives libpeano-claw: a radial dam break initialised through
the initialization callback, evolved with pyclaw_peano_evolveToTime and
gathered through the addPatchToSolution callback equals the direct batched
path bit for bit (every subgrid at the end time), and a lake at rest over a
bumpy bathymetry given as aux field stays exactly at rest."""
import numpy as np
import pytest

import pyclaw_ctypes as PC
from helpers import gpu_patchset, slab_for
from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S

pytestmark = pytest.mark.gpu


def _centers(px, py, sx, sy, n):
    hx, hy = sx / n, sy / n
    r = np.arange(n)
    return np.meshgrid((px + hx * r) + hx * 0.5, (py + hy * r) + hy * 0.5, indexing="ij")


def test_dam_break_through_the_c_interface_equals_the_direct_path():
    lib = PC.load()

    def init(q, qbc, aux, n0, n1, n2, nq, naux, sx, sy, sz, px, py, pz, skip):
        X, Y = _centers(px, py, sx, sy, n0)
        r = np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2)
        q[0] = np.where(r <= 0.15, 2.0, 1.0)
        q[1:] = 0.0
        return 1.0 / 9

    init_cb = PC.INIT(init)
    got = []
    add_cb = PC.ADD(lambda q, qbc, g, sx, sy, sz, px, py, pz, t: got.append(((px, py), q.copy(), g, t)))
    h, rank = PC.new(lib, 1.0 / 9, 16, 0, 1e-3, init_cb, add_cb)
    assert h, lib.pyclaw_peano_lastError()
    try:
        assert rank == 0 and lib.pyclaw_peano_runWorker(h) == 0
        lib.pyclaw_peano_evolveToTime(0.01, h)
        lib.pyclaw_peano_evolveToTime(0.02, h)
        lib.pyclaw_peano_gatherSolution(h)
    finally:
        lib.pyclaw_peano_destroy(h)
    ps = S.radial_dam_break(npx=9, n=16)
    c = P.Context(slab_doubles=slab_for(ps), max_patches=len(ps) + 8, max_groups=1,
                  params=P.swe_params(g=9.81, cfl=0.5))
    try:
        ids = gpu_patchset(c, ps)
        c.set_group_max_dt(0, np.inf)
        c.set_group_end_time(0, 0.0, 0.01)
        c.run(200, P.PCG_MODE_BATCHED)
        c.set_group_end_time(0, 0.01, 0.02)
        c.run(200, P.PCG_MODE_BATCHED)
        assert c.group_times()[0] == 0.02
        ref = c.download_many(ids, int(ps.packed.size))
    finally:
        c.close()
    assert len(got) == 81
    by_pos = {tuple(np.round(ps.pos[p], 12)): p for p in range(len(ps))}
    for pos, q, g, t in got:
        assert g == 1 and t == 0.02
        p = by_pos[tuple(np.round(pos, 12))]
        o = ps.offsets[p]
        assert np.array_equal(q.ravel().view(np.int64), ref[o:o + q.size].view(np.int64)), pos


def test_lake_at_rest_with_bathymetry_through_the_c_interface():
    lib = PC.load()
    bathy = {}

    def init(q, qbc, aux, n0, n1, n2, nq, naux, sx, sy, sz, px, py, pz, skip):
        X, Y = _centers(px, py, sx, sy, n0)
        b = np.round(0.3 * np.exp(-((X - 0.4) ** 2 + (Y - 0.6) ** 2) / 0.01) * 64.0) / 64.0
        aux[0] = b
        bathy[(round(px, 12), round(py, 12))] = b.copy()
        q[0] = 1.0 - b
        q[1:] = 0.0
        return 0.25

    init_cb = PC.INIT(init)
    out = []
    add_cb = PC.ADD(lambda q, qbc, g, sx, sy, sz, px, py, pz, t: out.append(((px, py), q.copy(), t)))
    h, _ = PC.new(lib, 0.25, 12, 1, 1e-3, init_cb, add_cb)
    assert h, lib.pyclaw_peano_lastError()
    try:
        lib.pyclaw_peano_evolveToTime(0.05, h)
        lib.pyclaw_peano_gatherSolution(h)
    finally:
        lib.pyclaw_peano_destroy(h)
    assert len(out) == 16
    for pos, q, t in out:
        b = bathy[(round(pos[0], 12), round(pos[1], 12))]
        assert t == 0.05
        assert np.all(q[0] + b == 1.0)
        assert np.all(q[1:] == 0.0)
