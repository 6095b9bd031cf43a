"""pcg_run_async + pcg_run_wait against pcg_run: the same dts and patch
vectors bit for bit; calls made between the two are ordered after the run on
the context's stream (a download sees the state after the run, an upload
lands after it); the calls that would start steps are refused while a run is
pending."""
import numpy as np
import pytest

from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S

from helpers import gpu_patchset, slab_for

pytestmark = pytest.mark.gpu

PRM = P.swe_params(g=9.81, cfl=0.5)


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def _ctx(ps):
    return P.Context(slab_doubles=slab_for(ps), max_patches=len(ps) + 16, max_groups=1, params=PRM)


def test_async_run_equals_run():
    ps = S.uneven_patches(grid=8)
    out = []
    for use_async in (False, True):
        ctx = _ctx(ps)
        try:
            ids = gpu_patchset(ctx, ps)
            ctx.set_group_max_dt(0, 1e9)
            rec = []
            for k in (3, 5):
                if use_async:
                    ctx.run_async(k)
                    # a download between the halves waits for the run
                    rec.append(_bits(ctx.download_many(ids, int(ps.packed.size))))
                    rec.append(list(ctx.run_wait()[:, 0]))
                else:
                    hist = ctx.run(k)
                    rec.append(_bits(ctx.download_many(ids, int(ps.packed.size))))
                    rec.append(list(hist[:, 0]))
            rec.append(ctx.stats()[0])
            out.append(rec)
        finally:
            ctx.close()
    sync, asyn = out
    for a, b in zip(sync, asyn):
        if isinstance(a, np.ndarray):
            assert np.array_equal(a, b)
        else:
            assert a == b


def test_async_dts_equal_run_dts():
    ps = S.uneven_patches(grid=6)
    dts = []
    for use_async in (False, True):
        ctx = _ctx(ps)
        try:
            gpu_patchset(ctx, ps)
            ctx.set_group_max_dt(0, 1e9)
            if use_async:
                ctx.run_async(6)
                dts.append(list(ctx.run_wait()[:, 0]))
            else:
                dts.append(list(ctx.run(6)[:, 0]))
        finally:
            ctx.close()
    assert dts[0] == dts[1]


def test_calls_that_step_are_refused_while_pending():
    ps = S.uneven_patches(grid=4)
    ctx = _ctx(ps)
    try:
        ids = gpu_patchset(ctx, ps)
        ctx.set_group_max_dt(0, 1e9)
        ctx.run_async(2)
        for call in (lambda: ctx.run(1), lambda: ctx.run_async(1), lambda: ctx.step(),
                     lambda: ctx.profile_step(), lambda: ctx.autotune(1),
                     lambda: ctx.set_time_stepping(P.TS_LOCAL)):
            with pytest.raises(P.PcgError):
                call()
        # an upload between the halves lands after the run: the state is the
        # uploaded one afterwards
        ctx.upload_many(ids, ps.packed)
        ctx.run_wait()
        got = ctx.download_many(ids, int(ps.packed.size))
        assert np.array_equal(_bits(got), _bits(ps.packed))
        with pytest.raises(P.PcgError):
            ctx.run_wait()
    finally:
        ctx.close()
