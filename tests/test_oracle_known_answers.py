"""The oracle against the reference's own known-answer tests.

Each test restates the setup of a registered reference test (file:line) and
checks the values that test validates.  The reference runs these through the
GhostLayerCompositor with NumericsTestStump (1 unknown, Default* strategies);
the compositor's face functor issues exactly the interpolateSolution call that
is made directly here (GhostlayerCompositorFunctors.cpp:23-72).
"""
import numpy as np
import pytest

from oracle import oracle as O


def _coarse_patch_for_interp(pos):
    # createPatch(1 unknown, 0, 0, subdivision 2, ghost 1, pos, size 3, level 0,
    #             time 0, dt 1)   GhostLayerCompositorTest.cpp:140-153
    p = O.Patch(2, ghost=1, nq=1, np_wo=0, np_w=0, pos=pos, size=3.0, level=0, time=0.0, dt=1.0)
    # uNew = 1 everywhere, uOld (incl. ghost) = -1, interior uOld 6,7,10,11 (:172-191)
    p.unew()[:] = 1.0
    p.uold()[:] = -1.0
    for (x, y, v) in [(0, 0, 6.0), (0, 1, 7.0), (1, 0, 10.0), (1, 1, 11.0)]:
        p.set_uold(x, y, 0, v)
    return p


def test_interpolation_coarse_to_fine_left_ghostlayer():
    """GhostLayerCompositorTest.cpp:126-216 (values :207-214)."""
    coarse = _coarse_patch_for_interp((2.0, 1.0))
    fine = O.Patch(2, ghost=2, nq=1, np_wo=0, np_w=0, pos=(5.0, 2.0), size=1.0, level=1,
                   time=0.0, dt=1.0 / 3.0)
    # face functor, source left of destination: faceSize (g=2, n=2), dstOffset (-2, 0)
    O.interpolate((2, 2), (-2, 0), coarse, fine, to_uold=True, to_current_time=False,
                  use_time_unew_or_uold=True)
    np.testing.assert_allclose(fine.get_uold(-2, 0), 65.0 / 9.0, rtol=1e-14)
    np.testing.assert_allclose(fine.get_uold(-2, 1), 67.0 / 9.0, rtol=1e-14)
    np.testing.assert_allclose(fine.get_uold(-1, 0), 73.0 / 9.0, rtol=1e-14)
    np.testing.assert_allclose(fine.get_uold(-1, 1), 25.0 / 3.0, rtol=1e-14)


def test_interpolation_coarse_to_fine_right_ghostlayer():
    """GhostLayerCompositorTest.cpp:218-307 (values :299-305)."""
    coarse = _coarse_patch_for_interp((2.0, 1.0))
    fine = O.Patch(2, ghost=2, nq=1, np_wo=0, np_w=0, pos=(1.0, 1.0), size=1.0, level=1,
                   time=0.0, dt=1.0 / 3.0)
    # source right of destination: dstOffset (subdivision, 0)
    O.interpolate((2, 2), (2, 0), coarse, fine, to_uold=True, to_current_time=False,
                  use_time_unew_or_uold=True)
    np.testing.assert_allclose(fine.get_uold(2, 0), 29.0 / 9.0, rtol=1e-14)
    np.testing.assert_allclose(fine.get_uold(2, 1), 31.0 / 9.0, rtol=1e-14)
    np.testing.assert_allclose(fine.get_uold(3, 0), 37.0 / 9.0, rtol=1e-14)
    np.testing.assert_allclose(fine.get_uold(3, 1), 13.0 / 3.0, rtol=1e-14)


@pytest.mark.parametrize("p1,s1,p2,s2,expected", [
    # GridLevelTransferTest.cpp:275-288, :290-304, :306-319
    ((0.5, 0.5), (5.0, 5.0), (1.0, 4.0), (1.5, 2.0), 2.25),
    ((1.0, 1.0), (1.0, 1.0), (2.0, 1.5), (1.0, 1.0), 0.0),
    ((-1.0, -1.0), (3.0, 3.0), (0.0, 3.0), (5.0, 5.0), 0.0),
])
def test_overlapping_region(p1, s1, p2, s2, expected):
    got = O.lib().pco_overlap_area(O.dvec(p1), O.dvec(s1), O.dvec(p2), O.dvec(s2))
    assert got == pytest.approx(expected, abs=1e-14)


def _regions(lower, upper, pos, size, sub, n):
    import ctypes as C
    off = (C.c_int * 8)()
    sz = (C.c_int * 8)()
    nr = O.lib().pco_regions_overlapped_by_ghostlayers(
        O.dvec(lower), O.dvec(upper), O.dvec(pos), O.dvec(size), O.dvec(sub),
        O.ivec(n), off, sz)
    return nr, [((off[2 * r], off[2 * r + 1]), (sz[2 * r], sz[2 * r + 1])) for r in range(4)]


def test_restriction_with_overlapping_bounds():
    """GhostLayerCompositorTest.cpp:624-657."""
    nr, regs = _regions((1.0, 1.0), (1.1, 1.1), (0.0, 0.0), (2.2, 2.2), (0.11, 0.11), (20, 20))
    assert regs[0] == ((0, 0), (20, 20))
    for r in regs[1:]:
        assert r == ((0, 0), (0, 0))


def test_partial_restriction_regions():
    """GhostLayerCompositorTest.cpp:659-700."""
    lo = 1.8 + 1e-13
    nr, regs = _regions((lo, lo), (1.2, 1.2), (1.0, 1.0), (1.0, 1.0), (0.1, 0.1), (10, 10))
    assert nr == 4
    assert regs[0] == ((0, 0), (2, 10))
    assert regs[1] == ((8, 0), (2, 10))
    assert regs[2] == ((2, 0), (6, 2))
    assert regs[3] == ((2, 8), (6, 2))


def test_partial_restriction_regions_with_infinite_lower_bounds():
    """GhostLayerCompositorTest.cpp:702-745."""
    big = np.finfo(np.float64).max
    upper = (4.0 / 27.0, 6.0 / 27.0 + 1.0 / 27.0 / 6.0)
    pos = (4.0 / 27.0, 2.0 / 9.0)
    sub = 1.0 / 27.0 / 6.0
    nr, regs = _regions((big, big), upper, pos, (1.0 / 27.0,) * 2, (sub, sub), (6, 6))
    assert regs[0] == ((0, 0), (0, 6))
    assert regs[1] == ((6, 0), (0, 6))
    assert regs[2] == ((0, 0), (6, 1))
    assert regs[3] == ((0, 6), (6, 0))


# GridLevelTransferTest::testRestrictionToVirtualPatch (GridLevelTransferTest.cpp:321-512):
# a fine leaf (3 x 3 cells, 1 unknown, ghost 2, at (1/3, 1/3), size 1/3) is
# restricted into a virtual coarse patch (2 x 2 cells on [0,1]^2), whose values
# then fill the ghost layer (width 2) of the coarse neighbour at (1, 0).
# The expected values (:495-501) weigh the fine cells that overlap one virtual
# cell by regionFraction * (1, 1/2, 1/2, 1/4) and combine each fine cell's
# uNew n and uOld o as tf * n + (1 - tf) * o with tf = 2 for ghost cell (-2, 0)
# and tf = 4/3 for (-2, 1), (-1, 0), (-1, 1).  In the reference those factors
# come out of GridLevelTransfer::stepDown / stepUp (Peano vertices, the
# virtual-patch life cycle, outside the path).  Here the fine interval is
# [0, 1], so that DefaultRestriction's factors for the virtual times 0 and 1
# are 0 and 1 (the virtual patch holds the restricted uOld and uNew), and the
# neighbour's uNew time is the factor of the transfer from the virtual source
# (DefaultTransfer.cpph:29-41): 2 (time 1, dt 1) or 4/3 (time 1, dt 1/3).
RESTR_RF = (1.0 / 9.0) * (1.0 / 9.0) / (1.0 / 2.0) / (1.0 / 2.0)
RESTR_EXPECTED = {
    (-2, 0): RESTR_RF * (-1.0 * 9.0 + 1.0 / 2.0 * (2.0 - 1.0 * 8.0) + 1.0 / 2.0 * (2.0 * 3.0 - 1.0 * 6.0)
                         + 1.0 / 4.0 * (2.0 * 4.0 - 1.0 * 5.0)),
    (-2, 1): RESTR_RF * (4.0 / 3.0 * 2.0 - 1.0 / 3.0 * 7.0 + 1.0 / 2.0 * (4.0 / 3.0 - 1.0 / 3.0 * 8.0)
                         + 1.0 / 2.0 * (4.0 / 3.0 * 5.0 - 1.0 / 3.0 * 4.0)
                         + 1.0 / 4.0 * (4.0 / 3.0 * 4.0 - 1.0 / 3.0 * 5.0)),
    (-1, 0): RESTR_RF * (4.0 / 3.0 * 6.0 - 1.0 / 3.0 * 3.0 + 1.0 / 2.0 * (4.0 / 3.0 * 3.0 - 1.0 / 3.0 * 6.0)
                         + 1.0 / 2.0 * (4.0 / 3.0 * 7.0 - 1.0 / 3.0 * 2.0)
                         + 1.0 / 4.0 * (4.0 / 3.0 * 4.0 - 1.0 / 3.0 * 5.0)),
    (-1, 1): RESTR_RF * (4.0 / 3.0 * 8.0 - 1.0 / 3.0 + 1.0 / 2.0 * (4.0 / 3.0 * 5.0 - 1.0 / 3.0 * 4.0)
                         + 1.0 / 2.0 * (4.0 / 3.0 * 7.0 - 1.0 / 3.0 * 2.0)
                         + 1.0 / 4.0 * (4.0 / 3.0 * 4.0 - 1.0 / 3.0 * 5.0)),
}
# neighbour time intervals (time, dt) giving the transfer factor of each check
RESTR_NEIGHBOUR_TIME = {(-2, 0): (1.0, 1.0), (-2, 1): (1.0, 1.0 / 3.0), (-1, 0): (1.0, 1.0 / 3.0),
                        (-1, 1): (1.0, 1.0 / 3.0)}


def restriction_test_fine_values():
    """uNew (x, y) = 3x + y and uOld (x, y) = 9 - (3x + y), :396-431."""
    return [(x, y, 3.0 * x + y, 9.0 - (3.0 * x + y)) for x in range(3) for y in range(3)]


def test_restriction_to_virtual_patch():
    """GridLevelTransferTest.cpp:321-512 (values :495-501) on the oracle."""
    for (gx, gy), expected in RESTR_EXPECTED.items():
        fine = O.Patch(3, ghost=2, nq=1, np_wo=0, np_w=0, pos=(1.0 / 3.0, 1.0 / 3.0), size=1.0 / 3.0,
                       level=1, time=0.0, dt=1.0)
        for x, y, n, o in restriction_test_fine_values():
            fine.set_unew(x, y, 0, n)
            fine.set_uold(x, y, 0, o)
        virtual = O.Patch(2, ghost=2, nq=1, np_wo=0, np_w=0, pos=(0.0, 0.0), size=1.0, level=0,
                          is_leaf=False, is_virtual=True)
        O.restrict(fine, virtual, only_overlapped=False, swe=False)
        t, dt = RESTR_NEIGHBOUR_TIME[(gx, gy)]
        neighbour = O.Patch(2, ghost=2, nq=1, np_wo=0, np_w=0, pos=(1.0, 0.0), size=1.0, level=0,
                            time=t, dt=dt)
        O.transfer_ghostlayer((2, 2), (0, 0), (-2, 0), virtual, neighbour)
        assert neighbour.get_uold(gx, gy) == pytest.approx(expected, rel=1e-13, abs=1e-15)
