"""The synthetic inputs follow the configurations' definitions (no GPU):
sizes, seeds, value distributions and boundary conditions of the radial dam
break (config 1), the 3-level breaking dam (config 2), the uneven mosaic
(config 3, at 64 x 64 slots; the bench's 224 x 224 mosaic draws from the
same generator), the coastal tsunami (config 5) and the request stream of
the serving form (config 4)."""
import numpy as np
import pytest

from peanoclaw_gb300 import scenarios as S
from peanoclaw_gb300 import serving as SV


def test_radial_dam_break_9x9_patches_of_16x16():
    ps = S.radial_dam_break(npx=9, n=16)
    assert len(ps) == 81 and set(ps.n) == {16} and ps.cells() == 20736
    for p in range(len(ps)):
        unew, _, b = ps.views(p)
        X, Y = S._centers(ps.pos[p], ps.size[p], 16, ghost=False)
        r = np.hypot(X - 0.5, Y - 0.5)
        assert np.array_equal(unew[0], np.where(r <= 0.15, 2.0, 1.0))
        assert not unew[1].any() and not unew[2].any() and not b.any()
    # reflecting walls on the four domain faces, nowhere inside
    w = np.array(ps.wall).reshape(9, 9)
    assert (w[0, :] & 1).all() and (w[-1, :] & 2).all() and (w[:, 0] & 4).all() and (w[:, -1] & 8).all()
    assert not w[1:-1, 1:-1].any()


def test_breaking_dam_three_levels():
    ps = S.breaking_dam_amr(base=9, n=27, levels=3)
    leaves = [p for p in range(len(ps)) if ps.leaf[p]]
    assert len(ps) == 1539 and len(leaves) == 1377 and set(ps.n) == {27}
    # 3x refinement: patch edges 1/9, 1/27, 1/81 of the domain; the finest
    # level sits on the dam (x = 0.5)
    sizes = sorted({round(ps.size[p][0] * 81) for p in range(len(ps))})
    assert sizes == [1, 3, 9]
    fine = [p for p in leaves if round(ps.size[p][0] * 81) == 1]
    assert fine and all(abs(ps.pos[p][0] + 0.5 / 81 - 0.5) < 0.1 for p in fine)
    for p in leaves:
        unew, _, b = ps.views(p)
        X, Y = S._centers(ps.pos[p], ps.size[p], 27, ghost=True)
        # h = 1 left of the dam, 0.5 right of it, at rest
        assert np.array_equal(unew[0], np.where(X[1:-1, 1:-1] < 0.5, 1.0, 0.5))
        assert not unew[1].any() and not unew[2].any()
        # b = 0.2 exp(-|x - (0.7, 0.5)|^2 / (2 0.05^2)), ghost ring included
        bb = 0.2 * np.exp(-((X - 0.7) ** 2 + (Y - 0.5) ** 2) / (2.0 * 0.05 * 0.05))
        assert np.allclose(b, bb, rtol=0, atol=1e-15)


def test_uneven_mosaic_sizes_and_values():
    ps = S.uneven_patches(grid=64)
    n = np.array(ps.n)
    counts = np.array([np.count_nonzero(n == s) for s in (8, 16, 32, 64)])
    # sizes drawn uniformly from {8, 16, 32, 64} (about 1360 cells per patch)
    assert counts.sum() == 64 * 64
    assert np.all(np.abs(counts / counts.sum() - 0.25) < 0.03)
    assert abs(ps.cells() / len(ps) - 1360) < 60
    # about a fifth of the cells dry
    assert 0.1 < ps.meta["dry_fraction"] < 0.3
    for p in range(0, len(ps), 37):
        unew, _, b = ps.views(p)
        assert np.isfinite(b).all()
        assert not unew[1].any() and not unew[2].any()
        # h = max(0, 1 - b) + 0.1 U[-1, 1], clamped at 0
        h = unew[0]
        assert (h >= 0.0).all()
        assert np.all(np.abs(h - np.maximum(0.0, 1.0 - b[1:-1, 1:-1])) <= 0.1 + 1e-12)


def test_coastal_tsunami_has_dry_land_along_the_coast():
    ps = S.coastal_tsunami()
    leaves = [p for p in range(len(ps)) if ps.leaf[p]]
    assert len(set(ps.n)) == 1 and ps.n[0] == 27
    peak = 0.0
    for p in leaves:
        unew, _, b = ps.views(p)
        X, Y = S._centers(ps.pos[p], ps.size[p], 27, ghost=False)
        h = unew[0]
        assert (h >= 0.0).all() and not unew[1].any() and not unew[2].any()
        # the seafloor rises above the still surface in the last 5 % of the domain
        assert not h[X > 0.98].any()
        wet = h > 0.0
        if wet.any():
            peak = max(peak, float(np.max((h + b[1:-1, 1:-1])[wet])))
    # the surface hump of amplitude 0.5 over the still level 1 (wet cells)
    assert 1.45 < peak <= 1.5 + 1e-12


def test_request_stream():
    reqs = SV.make_requests(128, rate=8.0, seed=42, n=32, levels=(1, 3))
    arr = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(arr) > 0) and abs(np.mean(np.diff(arr)) - 1 / 8.0) < 0.25 / 8.0
    cells = np.array([r.cells for r in reqs], dtype=np.float64)
    assert cells.min() >= 1e4 and cells.max() <= 4e6
    # log-uniform sizes: the median near the geometric middle of the range
    assert abs(np.median(np.log(cells)) - 0.5 * (np.log(1e4) + np.log(4e6))) < 0.8
    lv = np.array([r.levels for r in reqs])
    assert set(lv.tolist()) == {1, 2, 3}
    assert all(0.2 < np.mean(lv == k) < 0.47 for k in (1, 2, 3))
    assert 0.35 < np.mean([r.kind == "dam_break" for r in reqs]) < 0.65
    assert all(0.05 <= r.t_end <= 0.5 for r in reqs)
