"""The oracle's FP32 twin (pco32_grid_step, the CPU baseline at the
reference's float precision) against the FP64 oracle: same dts and fields to
float rounding on the uneven mosaic (copies, coarse-fine interpolation,
walls, wet and dry cells), a lake at rest stays exactly at rest, and the time
intervals advance alike."""
import numpy as np

from helpers import oracle_params, oracle_patchset
from oracle import oracle as O
from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S

PRM = P.swe_params(g=9.81, cfl=0.5)


def _f32(pats):
    return [np.ascontiguousarray(p.u.astype(np.float32)) for p in pats]


def test_fp32_twin_follows_the_fp64_oracle_on_the_uneven_mosaic():
    ps = S.uneven_patches(grid=6, sizes=(8, 16, 32))
    assert any(int(it[0]) == 1 for it in ps.items)    # coarse-fine interpolation items
    prm = oracle_params(PRM)
    a = oracle_patchset(ps)
    b = oracle_patchset(ps)
    u32 = _f32(b)
    for step in range(6):
        dt64 = O.grid_step(a, ps.items, ps.wall, prm, np.inf, n_threads=2)[0]
        dt32 = O.grid_step_f32(b, u32, ps.items, ps.wall, prm, np.inf, n_threads=2)
        assert abs(dt32 - dt64) <= 1e-6 * dt64, (step, dt32, dt64)
    for p, q, u in zip(a, b, u32):
        n = p.nx * p.ny
        ref = p.u[: 3 * n].reshape(3, n)
        got = u[: 3 * n].reshape(3, n).astype(np.float64)
        h_scale = max(1.0, float(np.abs(ref[0]).max()))
        assert np.abs(got[0] - ref[0]).max() <= 2e-6 * h_scale
        m_scale = max(1e-3, float(np.abs(ref[1:]).max()))
        assert np.abs(got[1:] - ref[1:]).max() <= 5e-5 * m_scale
        assert abs(q.s.time - p.s.time) <= 1e-6 * max(p.s.time, 1e-12)
        assert abs(q.s.dt - p.s.dt) <= 1e-6 * p.s.dt


def test_fp32_twin_keeps_a_flat_lake_at_rest():
    ps = S.uneven_patches(grid=3, sizes=(8, 16))
    prm = oracle_params(PRM)
    b = oracle_patchset(ps)
    for p in b:
        n = p.nx * p.ny
        p.u[:] = 0.0
        p.u[:n] = 1.0                                  # h = 1 in uNew, b = 0, no momentum
    u32 = _f32(b)
    for _ in range(3):
        dt = O.grid_step_f32(b, u32, ps.items, ps.wall, prm, np.inf)
        assert dt > 0.0
    for p, u in zip(b, u32):
        n = p.nx * p.ny
        assert np.all(u[:n] == np.float32(1.0))
        assert np.all(u[n:3 * n] == 0.0)


def test_fp32_twin_threads_agree():
    ps = S.uneven_patches(grid=4, sizes=(8, 16, 32))
    prm = oracle_params(PRM)
    outs = []
    for threads in (1, 3):
        b = oracle_patchset(ps)
        u32 = _f32(b)
        for _ in range(3):
            O.grid_step_f32(b, u32, ps.items, ps.wall, prm, np.inf, n_threads=threads)
        outs.append(np.concatenate(u32))
    assert np.array_equal(outs[0].view(np.int32), outs[1].view(np.int32))
