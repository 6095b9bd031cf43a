"""VTU output from the device buffers (one gather of uNew and b) equals the
output written from the oracle's state after the same steps, cell by cell
and bit for bit; the batched time query matches the per-patch one."""
import numpy as np
import pytest

from helpers import gpu_patchset, oracle_params, oracle_patchset, slab_for
from oracle import oracle as O
from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S
from peanoclaw_gb300 import vtu

pytestmark = pytest.mark.gpu

PRM = P.swe_params(g=9.81, cfl=0.5)


def test_device_vtu_equals_oracle_vtu(tmp_path):
    ps = S.uneven_patches(grid=4, sizes=(8, 16, 32))
    c = P.Context(slab_doubles=slab_for(ps), max_patches=len(ps) + 8, max_groups=1, params=PRM)
    try:
        ids = gpu_patchset(c, ps)
        c.set_group_max_dt(0, 1e9)
        c.run(7, P.PCG_MODE_BATCHED)
        geo = [(ps.pos[p], ps.size[p], (ps.n[p], ps.n[p]), ps.level[p]) for p in range(len(ps))]
        recs = vtu.patch_records_from_context(c, ids, geo)
        t = c.times_of(ids)
        for k, pid in enumerate(ids):
            tt = c.get_time(int(pid))
            assert (t[k, 0], t[k, 1]) == (tt["time"], tt["dt"])
    finally:
        c.close()
    pats = oracle_patchset(ps)
    for _ in range(7):
        O.grid_step(pats, ps.items, ps.wall, oracle_params(PRM), 1e9)
    orec = [vtu.patch_record_from_vector(pats[p].u, ps.pos[p], ps.size[p], ps.n[p], ps.level[p],
                                         time=pats[p].s.time, dt=pats[p].s.dt) for p in range(len(ps))]
    fa, fb = str(tmp_path / "gpu.vtu"), str(tmp_path / "oracle.vtu")
    vtu.write_vtu(fa, recs)
    vtu.write_vtu(fb, orec)
    a, b = vtu.read_vtu(fa), vtu.read_vtu(fb)
    for name in ("q0", "q1", "q2", "pWG0", "timeOld", "timeNew"):
        assert np.array_equal(a[2][name].view(np.int64), b[2][name].view(np.int64)), name
    assert vtu.compare_cells(a, b) == (0, 0.0)
