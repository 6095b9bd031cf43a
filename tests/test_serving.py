"""Continuous batching: requests admitted while others run give the same
result alone and in the mix (bit for bit: groups share launches but each
group's dt and data are its own)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_results_identical_alone_and_in_the_mix():
    from peanoclaw_gb300 import serving as SV

    reqs = SV.make_requests(6, rate=200.0, seed=7, cells=(2e3, 3e4), t_end=(0.01, 0.03), n=16)
    srv = SV.Server(slab_doubles=4_000_000, max_groups=3, max_patches=4096)
    try:
        done, wall = srv.serve(reqs, max_wall=120.0)
    finally:
        srv.close()
    assert len(done) == len(reqs)
    # at least one request waited for a slot: admission is by free group/HBM
    assert max(r.admitted - r.arrival for r in done) >= 0.0
    by_id = {r.rid: r for r in done}
    for rid in (0, 3, 5):
        mixed = by_id[rid]
        alone = SV.run_alone(mixed, slab_doubles=2_000_000)
        assert alone.steps == mixed.steps
        assert np.array_equal(alone.result, mixed.result)
        assert np.all(np.isfinite(mixed.result))


def test_admission_refuses_when_hbm_is_full():
    from peanoclaw_gb300 import serving as SV

    big = SV.make_requests(1, rate=1.0, seed=3, cells=(3e4, 3e4), t_end=(0.01, 0.01), n=16)[0]
    srv = SV.Server(slab_doubles=50_000, max_groups=2, max_patches=256)
    try:
        assert not srv.admit(big, 0.0)   # does not fit into 50k doubles
        assert not srv.resident
    finally:
        srv.close()


def test_adaptive_requests_identical_alone_and_in_the_mix():
    """Requests with 2-3 levels of 3x refinement (interpolation, flux
    correction and restriction every step, remeshed every 8 of their own
    steps from the device criterion) next to uniform ones: each adaptive
    result -- its hierarchy and every patch vector in grid order -- is the
    same alone (one step per replay) and in the mix (8 steps per replay)."""
    from peanoclaw_gb300 import serving as SV

    reqs = SV.make_requests(6, rate=200.0, seed=12, cells=(2e4, 2e5), t_end=(0.01, 0.02), n=16,
                            levels=(1, 3))
    assert sorted(set(r.levels for r in reqs)) == [1, 2, 3]
    srv = SV.Server(slab_doubles=16_000_000, max_groups=3, max_patches=8192, steps_per_batch=8,
                    remesh_every=8)
    try:
        done, wall = srv.serve(reqs, max_wall=300.0)
        assert srv.remesh_s > 0.0
    finally:
        srv.close()
    assert len(done) == len(reqs)
    for mixed in done:
        if mixed.levels == 1 and mixed.rid % 2:
            continue
        alone = SV.run_alone(mixed, slab_doubles=8_000_000, remesh_every=8)
        assert alone.steps == mixed.steps
        assert alone.result.shape == mixed.result.shape
        assert np.array_equal(alone.result.view(np.int64), mixed.result.view(np.int64)), mixed.rid
        assert np.all(np.isfinite(mixed.result))
