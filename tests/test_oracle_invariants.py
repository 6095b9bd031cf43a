"""Invariants of the oracle's synchronous step that need no reference data
(CPU): the 9x9x16² radial dam break keeps its 4-fold symmetry (mirror in x
and in y, transpose; momenta mirror with a sign) to round-off, and with
reflecting walls and no flux correction the water volume stays constant to
round-off.  The CUDA path equals the oracle bit for bit, so both hold there
as well."""
import numpy as np

from helpers import oracle_params, oracle_patchset
from oracle import oracle as O
from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S

PRM = P.swe_params(g=9.81, cfl=0.5)


def _field(ps, pats, npx, n):
    out = np.zeros((3, npx * n, npx * n))
    for p, op in enumerate(pats):
        i, j = int(round(ps.pos[p][0] * npx)), int(round(ps.pos[p][1] * npx))
        out[:, i * n:(i + 1) * n, j * n:(j + 1) * n] = op.unew()
    return out


def test_radial_dam_break_stays_symmetric():
    npx, n = 9, 16
    ps = S.radial_dam_break(npx=npx, n=n)
    prm = oracle_params(PRM)
    pats = oracle_patchset(ps)
    for _ in range(40):
        O.grid_step(pats, ps.items, ps.wall, prm, np.inf)
    h, hu, hv = _field(ps, pats, npx, n)
    assert h.max() > 1.5 and np.abs(hu).max() > 1.0     # the wave has moved
    tol = 1e-13
    assert np.abs(h - h[::-1, :]).max() < tol
    assert np.abs(h - h[:, ::-1]).max() < tol
    assert np.abs(h - h.T).max() < tol
    assert np.abs(hu + hu[::-1, :]).max() < tol           # x momentum flips in x
    assert np.abs(hv + hv[:, ::-1]).max() < tol           # y momentum flips in y
    assert np.abs(hu - hv.T).max() < tol                  # transpose swaps them


def test_volume_is_conserved_with_reflecting_walls():
    npx, n = 9, 16
    ps = S.radial_dam_break(npx=npx, n=n)
    prm = oracle_params(PRM)
    pats = oracle_patchset(ps)
    cell = (1.0 / (npx * n)) ** 2
    v0 = sum(op.unew()[0].sum() for op in pats) * cell
    for _ in range(40):
        O.grid_step(pats, ps.items, ps.wall, prm, np.inf)
    v1 = sum(op.unew()[0].sum() for op in pats) * cell
    assert abs(v1 - v0) <= 1e-13 * v0
