"""Parity of the CUDA path (through the C ABI) with the oracle.

The CUDA kernels issue the same IEEE operations as the oracle, so every
comparison here is bit-exact (np.array_equal on the whole patch vector,
ghost layers and time intervals included).
"""
import numpy as np
import pytest

from oracle import oracle as O
from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S
from peanoclaw_gb300.numerics import DefaultNumerics, Patch, SWEKernel

from helpers import (gpu_patchset, oracle_params, oracle_patch_from, oracle_patchset,
                     random_swe_vector, slab_for)

pytestmark = pytest.mark.gpu

PRM = P.swe_params(g=9.81, cfl=0.5)


@pytest.fixture(scope="module")
def ctx():
    c = P.Context(slab_doubles=8_000_000, max_patches=4096, max_groups=4, params=PRM)
    yield c
    c.close()


def _bit_equal(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    same = (a == b) | (np.isnan(a) & np.isnan(b))
    # distinguish signed zeros as well
    same &= np.signbit(a) == np.signbit(b)
    return bool(np.all(same))


@pytest.mark.parametrize("n", [2, 8, 16, 27, 32, 64])
@pytest.mark.parametrize("kind", ["random", "lake", "dry"])
def test_solve_timestep_bit_exact(ctx, n, kind):
    """SWEKernel::solveTimestep on one patch: state, ghost layers, dt, times."""
    rng = np.random.default_rng(1000 + n)
    vec = random_swe_vector(rng, n, lake=(kind == "lake"), dry_fraction=0.6 if kind == "dry" else 0.2)
    pos, size = (0.25, 0.5), (0.125, 0.125)
    gp = Patch(ctx, n, pos, size)
    gp.upload(vec)
    gp.set_time_intervals(time=0.5, dt=0.01)
    num = SWEKernel(ctx)
    op = oracle_patch_from(vec.copy(), n, pos, size, time=0.5, dt=0.01)
    for max_dt in (1e-3, 1e9):
        dt_g, est_g = num.solveTimestep(gp, max_dt)
        dt_o, est_o = O.solve_timestep(op, oracle_params(PRM), max_dt)
        assert dt_g == dt_o and est_g == est_o
        assert _bit_equal(gp.download(), op.u)
        t = gp.get_time_intervals()
        assert t["time"] == op.s.time and t["dt"] == op.s.dt and t["est_next"] == op.s.est_next
    if kind == "lake":
        hu = op.unew()[1]
        assert np.all(hu == 0.0)
    ctx.free(gp.id)


def test_lake_at_rest_is_exactly_still(ctx):
    rng = np.random.default_rng(7)
    n = 32
    vec = random_swe_vector(rng, n, lake=True)
    gp = Patch(ctx, n, (0.0, 0.0), (1.0, 1.0))
    gp.upload(vec)
    num = SWEKernel(ctx)
    before = gp.download()
    for _ in range(5):
        num.copyUNewToUOld(gp)
        num.solveTimestep(gp, 1e-3)
    after = gp.download()
    a = 3 * n * n
    assert np.array_equal(after[:a], before[:a])
    ctx.free(gp.id)


@pytest.mark.parametrize("dim,up", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_fill_boundary_layer_bit_exact(ctx, dim, up):
    rng = np.random.default_rng(3)
    n = 12
    vec = random_swe_vector(rng, n)
    gp = Patch(ctx, n, (0.0, 0.0), (1.0, 1.0))
    gp.upload(vec)
    op = oracle_patch_from(vec.copy(), n)
    SWEKernel(ctx).fillBoundaryLayer(gp, dim, up)
    O.lib().pco_swe_fill_boundary_layer(op.ptr(), dim, up)
    assert _bit_equal(gp.download(), op.u)
    ctx.free(gp.id)


def _pair(ctx, rng, ns, nd, spos, ssize, dpos, dsize, nq=3, gs=1, gd=1, npw=1, stime=(0.0, 0.0),
          dtime=(0.0, 0.0)):
    vs = rng.normal(1.0, 0.3, P.vector_size(ns, gs, nq, 0, npw))
    vd = rng.normal(1.0, 0.3, P.vector_size(nd, gd, nq, 0, npw))
    gs_ = Patch(ctx, ns, spos, ssize, ghost=gs, unknowns=nq, params_with_ghost=npw)
    gd_ = Patch(ctx, nd, dpos, dsize, ghost=gd, unknowns=nq, params_with_ghost=npw)
    gs_.upload(vs)
    gd_.upload(vd)
    gs_.set_time_intervals(time=stime[0], dt=stime[1])
    gd_.set_time_intervals(time=dtime[0], dt=dtime[1])
    os_ = oracle_patch_from(vs.copy(), ns, spos, ssize, ghost=gs, nq=nq, np_w=npw, time=stime[0], dt=stime[1])
    od_ = oracle_patch_from(vd.copy(), nd, dpos, dsize, ghost=gd, nq=nq, np_w=npw, time=dtime[0], dt=dtime[1])
    return gs_, gd_, os_, od_


@pytest.mark.parametrize("times", [((0.0, 0.0), (0.0, 0.0)), ((1.0, 0.5), (1.25, 0.25)),
                                   ((0.3, 0.1), (0.3, 0.1))])
def test_transfer_ghostlayer_bit_exact(ctx, times):
    rng = np.random.default_rng(11)
    gs_, gd_, os_, od_ = _pair(ctx, rng, 10, 10, (0.0, 0.0), (1.0, 1.0), (1.0, 0.0), (1.0, 1.0),
                               stime=times[0], dtime=times[1])
    num = SWEKernel(ctx)
    num.transferGhostlayer((1, 10), (9, 0), (-1, 0), gs_, gd_)
    O.transfer_ghostlayer((1, 10), (9, 0), (-1, 0), os_, od_)
    num.transferGhostlayer((1, 1), (9, 9), (-1, -1), gs_, gd_)
    O.transfer_ghostlayer((1, 1), (9, 9), (-1, -1), os_, od_)
    assert _bit_equal(gd_.download(), od_.u)
    ctx.free(gs_.id)
    ctx.free(gd_.id)


@pytest.mark.parametrize("swe", [0, 1])
@pytest.mark.parametrize("to_uold,current,use_new", [(1, 0, 1), (0, 0, 1), (1, 1, 1), (0, 1, 0)])
def test_interpolation_bit_exact(ctx, swe, to_uold, current, use_new):
    rng = np.random.default_rng(21)
    # coarse source (9 cells of 1/27) left of a fine destination (27 cells of 1/81)
    gs_, gd_, os_, od_ = _pair(ctx, rng, 9, 27, (0.0, 0.0), (1.0 / 3, 1.0 / 3), (1.0 / 3, 1.0 / 9),
                               (1.0 / 9, 1.0 / 9), stime=(0.5, 0.2), dtime=(0.55, 0.05))
    num = SWEKernel(ctx) if swe else DefaultNumerics(ctx)
    if to_uold:
        size, off = (1, 27), (-1, 0)
    else:
        size, off = (27, 27), (0, 0)
    num.interpolateSolution(size, off, gs_, gd_, bool(to_uold), bool(current), bool(use_new))
    O.interpolate(size, off, os_, od_, to_uold=bool(to_uold), to_current_time=bool(current),
                  use_time_unew_or_uold=bool(use_new), swe=bool(swe))
    assert _bit_equal(gd_.download(), od_.u)
    assert _bit_equal(gs_.download(), os_.u)
    ctx.free(gs_.id)
    ctx.free(gd_.id)


def test_interpolation_reference_known_answers_on_gpu(ctx):
    """GhostLayerCompositorTest.cpp:126-216 through the CUDA path."""
    num = DefaultNumerics(ctx)
    coarse = Patch(ctx, 2, (2.0, 1.0), 3.0, ghost=1, unknowns=1, params_with_ghost=0)
    fine = Patch(ctx, 2, (5.0, 2.0), 1.0, level=1, ghost=2, unknowns=1, params_with_ghost=0)
    vc = np.full(coarse.vector_size, -1.0)
    vc[:4] = 1.0
    uold = vc[4:4 + 16].reshape(4, 4)
    uold[1, 1], uold[1, 2], uold[2, 1], uold[2, 2] = 6.0, 7.0, 10.0, 11.0
    vc[4 + 16:] = 0.0
    coarse.upload(vc)
    coarse.set_time_intervals(time=0.0, dt=1.0)
    fine.upload(np.zeros(fine.vector_size))
    fine.set_time_intervals(time=0.0, dt=1.0 / 3.0)
    num.interpolateSolution((2, 2), (-2, 0), coarse, fine, True, False, True)
    v = fine.download()
    uo = v[4:4 + 36].reshape(6, 6)
    np.testing.assert_allclose([uo[0, 2], uo[0, 3], uo[1, 2], uo[1, 3]],
                               [65 / 9, 67 / 9, 73 / 9, 25 / 3], rtol=1e-14)
    ctx.free(coarse.id)
    ctx.free(fine.id)


def test_restriction_to_virtual_patch_known_answers_on_gpu(ctx):
    """GridLevelTransferTest.cpp:321-512 (values :495-501) through the CUDA
    path: restriction of the fine leaf into the virtual patch, then the ghost
    transfer from the virtual patch into its coarse neighbour (the set-up and
    the time intervals of test_oracle_known_answers.test_restriction_to_virtual_patch);
    every value bit-exact against the oracle and within 1e-13 of the
    reference's expected value."""
    from test_oracle_known_answers import (RESTR_EXPECTED, RESTR_NEIGHBOUR_TIME,
                                           restriction_test_fine_values)
    num = DefaultNumerics(ctx)
    for (gx, gy), expected in RESTR_EXPECTED.items():
        fine = Patch(ctx, 3, (1.0 / 3.0, 1.0 / 3.0), 1.0 / 3.0, level=1, ghost=2, unknowns=1,
                     params_with_ghost=0)
        virtual = Patch(ctx, 2, (0.0, 0.0), 1.0, ghost=2, unknowns=1, params_with_ghost=0, leaf=False,
                        virtual=True)
        nb = Patch(ctx, 2, (1.0, 0.0), 1.0, ghost=2, unknowns=1, params_with_ghost=0)
        of = O.Patch(3, ghost=2, nq=1, np_wo=0, np_w=0, pos=(1.0 / 3.0, 1.0 / 3.0), size=1.0 / 3.0,
                     level=1, time=0.0, dt=1.0)
        for x, y, n, o in restriction_test_fine_values():
            of.set_unew(x, y, 0, n)
            of.set_uold(x, y, 0, o)
        ov = O.Patch(2, ghost=2, nq=1, np_wo=0, np_w=0, pos=(0.0, 0.0), size=1.0, is_leaf=False,
                     is_virtual=True)
        t, dt = RESTR_NEIGHBOUR_TIME[(gx, gy)]
        on = O.Patch(2, ghost=2, nq=1, np_wo=0, np_w=0, pos=(1.0, 0.0), size=1.0, time=t, dt=dt)
        fine.upload(of.u)
        fine.set_time_intervals(time=0.0, dt=1.0)
        virtual.upload(np.zeros(virtual.vector_size))
        nb.upload(np.zeros(nb.vector_size))
        nb.set_time_intervals(time=t, dt=dt)
        num.restrictSolution(fine, virtual, False)
        num.transferGhostlayer((2, 2), (0, 0), (-2, 0), virtual, nb)
        O.restrict(of, ov, only_overlapped=False, swe=False)
        O.transfer_ghostlayer((2, 2), (0, 0), (-2, 0), ov, on)
        assert _bit_equal(virtual.download(), ov.u)
        got = nb.download()
        assert _bit_equal(got, on.u)
        uo = got[4:4 + 36].reshape(6, 6)
        assert uo[gx + 2, gy + 2] == pytest.approx(expected, rel=1e-13, abs=1e-15)
        for p in (fine, virtual, nb):
            ctx.free(p.id)


@pytest.mark.parametrize("only_overlapped", [0, 1])
@pytest.mark.parametrize("swe", [0, 1])
def test_restriction_bit_exact(ctx, only_overlapped, swe):
    rng = np.random.default_rng(31)
    # fine leaf (27^2 cells of 1/243) inside a virtual coarse patch (27^2 of 1/81)
    gs_, gd_, os_, od_ = _pair(ctx, rng, 27, 27, (1.0 / 9, 2.0 / 9), (1.0 / 9, 1.0 / 9),
                               (0.0, 0.0), (1.0 / 3, 1.0 / 3), stime=(0.2, 0.05))
    rl, ru = (0.12, 0.25), (0.2, 0.3)
    gd_.set_time_intervals(time=0.0, dt=0.0, restr_lower=rl, restr_upper=ru)
    od_.s.restr_lower[0], od_.s.restr_lower[1] = rl
    od_.s.restr_upper[0], od_.s.restr_upper[1] = ru
    num = SWEKernel(ctx) if swe else DefaultNumerics(ctx)
    num.restrictSolution(gs_, gd_, bool(only_overlapped))
    O.restrict(os_, od_, only_overlapped=bool(only_overlapped), swe=bool(swe))
    if swe:
        num.postProcessRestriction(gd_)
        O.lib().pco_swe_post_process_restriction(od_.ptr())
    assert _bit_equal(gd_.download(), od_.u)
    ctx.free(gs_.id)
    ctx.free(gd_.id)


@pytest.mark.parametrize("dim,direction", [(0, 1), (0, -1), (1, 1), (1, -1)])
def test_flux_correction_bit_exact(ctx, dim, direction):
    rng = np.random.default_rng(41 + dim)
    ns, nd = 9, 9
    # fine source next to a coarse destination
    if dim == 0:
        spos = (1.0 / 3 - 1.0 / 9, 1.0 / 9) if direction == 1 else (1.0 / 3, 1.0 / 9)
        dpos = (1.0 / 3, 0.0) if direction == 1 else (0.0, 0.0)
    else:
        spos = (1.0 / 9, 1.0 / 3 - 1.0 / 9) if direction == 1 else (1.0 / 9, 1.0 / 3)
        dpos = (0.0, 1.0 / 3) if direction == 1 else (0.0, 0.0)
    gs_, gd_, os_, od_ = _pair(ctx, rng, ns, nd, spos, (1.0 / 9, 1.0 / 9), dpos, (1.0 / 3, 1.0 / 3),
                               stime=(0.1, 0.02), dtime=(0.1, 0.06))
    num = SWEKernel(ctx)
    for p_g, p_o in ((gs_, os_), (gd_, od_)):
        num.computeFluxes(p_g)
        O.lib().pco_compute_fluxes(p_o.ptr(), 1.0)
    num.applyFluxCorrection(gs_, gd_, dim, direction)
    O.lib().pco_apply_flux_correction(os_.ptr(), od_.ptr(), dim, direction)
    assert _bit_equal(gs_.download(), os_.u)
    assert _bit_equal(gd_.download(), od_.u)
    ctx.free(gs_.id)
    ctx.free(gd_.id)


def _grid_run(ps, steps, mode, max_dt=1e9, oracle_steps=None):
    c = P.Context(slab_doubles=slab_for(ps), max_patches=len(ps) + 8, max_groups=1, params=PRM)
    ids = gpu_patchset(c, ps)
    c.set_group_max_dt(0, max_dt)
    if mode == "step":
        dts = [c.step(P.PCG_MODE_BATCHED)[0] for _ in range(steps)]
    elif mode == "plain":
        dts = list(c.run(steps, P.PCG_MODE_PLAIN)[:, 0])
    else:
        dts = list(c.run(steps, P.PCG_MODE_BATCHED)[:, 0])
    total = int(ps.packed.size)
    out = c.download_many(ids, total)
    times = [c.get_time(i) for i in ids[:3]]
    c.close()
    pats = oracle_patchset(ps)
    odts = []
    for _ in range(steps):
        odts.append(O.grid_step(pats, ps.items, ps.wall, oracle_params(PRM), max_dt)[0])
    oout = np.concatenate([p.u for p in pats])
    return out, dts, oout, odts, times, pats


@pytest.mark.parametrize("mode", ["step", "plain", "batched"])
def test_radial_dam_break_grid_bit_exact(mode):
    """The small CPU-runnable configuration: 9x9 patches of 16x16 cells,
    radial dam break, reflecting walls, g = 9.81, CFL 0.5, 100 steps."""
    ps = S.radial_dam_break(npx=9, n=16)
    steps = 100 if mode != "step" else 10
    out, dts, oout, odts, times, pats = _grid_run(ps, steps, mode)
    assert dts == odts
    assert _bit_equal(out, oout)
    assert times[0]["time"] == pats[0].s.time and times[0]["dt"] == pats[0].s.dt


def test_uneven_mosaic_bit_exact():
    """Mixed patch sizes (copy + interpolation faces), wet/dry bathymetry."""
    ps = S.uneven_patches(grid=6, sizes=(8, 16, 32))
    assert ps.meta["dry_fraction"] > 0.05
    out, dts, oout, odts, _, _ = _grid_run(ps, 40, "batched")
    assert dts == odts
    assert np.all(np.isfinite(out))
    assert _bit_equal(out, oout)


def test_mass_conservation_closed_basin():
    """Reflecting walls, flat bottom, no dry cells: mass is conserved to round-off."""
    ps = S.radial_dam_break(npx=5, n=16)
    c = P.Context(slab_doubles=slab_for(ps), max_patches=len(ps) + 8, max_groups=1, params=PRM)
    ids = gpu_patchset(c, ps)

    def mass():
        v = c.download_many(ids, int(ps.packed.size))
        tot = 0.0
        for p in range(len(ps)):
            o = ps.offsets[p]
            n = ps.n[p]
            tot += v[o:o + n * n].sum() * (ps.size[p][0] / n) * (ps.size[p][1] / n)
        return tot
    m0 = mass()
    c.run(200, P.PCG_MODE_BATCHED)
    m1 = mass()
    c.close()
    assert abs(m1 - m0) / m0 < 1e-13


def test_integer_pipe_divide_and_sqrt_match_ieee(ctx):
    """The sweep's divide / square root (integer pipes) equal the hardware
    IEEE results bit for bit on 2^26 pseudo-random operand pairs."""
    assert ctx.check_ieee_emulation(1 << 26, seed=20261203) == 0
