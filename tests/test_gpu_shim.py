"""The compiled GPU Numerics plugin driven through its virtuals, in the order
of a Peano grid iteration (compositor transfers and interpolations, then per
subgrid copyUNewToUOld, the domain boundary layers, solveTimestep with the
global timestep bound, getDemandedMeshWidth), against the same call sequence
on the oracle: dts, CFL estimates, demanded mesh widths and every patch
vector bit for bit."""
import ctypes as C

import numpy as np
import pytest

import shim_build
from helpers import oracle_criterion, oracle_params, oracle_patchset
from oracle import oracle as O
from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S

pytestmark = pytest.mark.gpu

PRM = P.swe_params(g=9.81, cfl=0.5)


def _drive(ps, steps, max_dt, tmp_path):
    lib = C.CDLL(shim_build.build(str(tmp_path)))
    f = lib.shim_drive_iterations
    f.restype = C.c_int
    lib.shim_last_error.restype = C.c_char_p
    n = len(ps)
    ctx = P.Context(slab_doubles=int(ps.packed.size * 1.2) + 4096, max_patches=n + 8, max_groups=1, params=PRM)
    try:
        ids = np.array([ctx.alloc(ps.n[p], pos=ps.pos[p], size=ps.size[p]) for p in range(n)], dtype=np.int32)
        ctx.upload_many(ids, ps.packed)
        pos = np.ascontiguousarray(np.array(ps.pos, dtype=np.float64))
        size = np.ascontiguousarray(np.array(ps.size, dtype=np.float64))
        sub = np.ascontiguousarray(np.array(ps.n, dtype=np.int32))
        walls = np.ascontiguousarray(np.array(ps.wall, dtype=np.uint8))
        items = np.ascontiguousarray(np.asarray(ps.items, dtype=np.int32).reshape(-1, 9))
        dt = np.zeros((steps, n))
        est = np.zeros((steps, n))
        width = np.zeros((steps, n))
        ptr = lambda a, t: a.ctypes.data_as(C.POINTER(t))
        rc = f(ctx.h, n, ptr(ids, C.c_int32), ptr(pos, C.c_double), ptr(size, C.c_double), ptr(sub, C.c_int32),
               ptr(walls, C.c_uint8), len(items), ptr(items, C.c_int32), steps, C.c_double(max_dt),
               ptr(dt, C.c_double), ptr(est, C.c_double), ptr(width, C.c_double))
        assert rc == 0, lib.shim_last_error()
        out = ctx.download_many(ids, int(ps.packed.size))
    finally:
        ctx.close()
    return out, dt, est, width


def _oracle(ps, steps, max_dt):
    prm = oracle_params(PRM)
    pats = oracle_patchset(ps)
    n = len(ps)
    dt = np.zeros((steps, n))
    est = np.zeros((steps, n))
    width = np.zeros((steps, n))
    for s in range(steps):
        for it in np.asarray(ps.items).reshape(-1, 9):
            kind, src, dst = int(it[0]), int(it[1]), int(it[2])
            if kind == P.PCG_GHOST_COPY:
                O.transfer_ghostlayer((it[3], it[4]), (it[5], it[6]), (it[7], it[8]), pats[src], pats[dst])
            else:
                O.interpolate((it[3], it[4]), (it[7], it[8]), pats[src], pats[dst], to_uold=True,
                              to_current_time=False, use_time_unew_or_uold=True, swe=True)
        for p in range(n):
            q = pats[p]
            O.lib().pco_copy_unew_to_uold(q.ptr())
            for bit, (d, up) in ((1, (0, 0)), (8, (1, 1)), (2, (0, 1)), (4, (1, 0))):
                if ps.wall[p] & bit:
                    O.lib().pco_swe_fill_boundary_layer(q.ptr(), d, up)
            dt[s, p], est[s, p] = O.solve_timestep(q, prm, max_dt)
            g = oracle_criterion(q, 0)
            width[s, p] = 1.0 / 243.0 if g > 0.1 else (1.0 / 27.0 if g < 0.1 else q.s.size[0] / q.s.nx)
    return np.concatenate([q.u for q in pats]), dt, est, width


@pytest.mark.parametrize("case", ["radial_dam_break_9x9x16", "uneven_mosaic"])
def test_plugin_iterations_match_the_oracle(case, tmp_path):
    if case == "radial_dam_break_9x9x16":
        ps, steps, max_dt = S.radial_dam_break(npx=9, n=16), 10, 2e-4
    else:
        ps, steps, max_dt = S.uneven_patches(grid=4), 4, 1e-4
    got, dt, est, width = _drive(ps, steps, max_dt, tmp_path)
    ref, odt, oest, owidth = _oracle(ps, steps, max_dt)
    assert np.array_equal(dt, odt) and np.array_equal(est, oest) and np.array_equal(width, owidth)
    # the global timestep bound is below every subgrid's CFL timestep:
    # a synchronous step of every subgrid
    assert np.all(dt == max_dt)
    assert np.array_equal(got.view(np.int64), ref.view(np.int64))
