"""VTU output (VTUSubgridPlotter's cells and data): written, read back bit for
bit, and compared cell by cell the way compareResult.py does."""
import numpy as np

from peanoclaw_gb300 import scenarios as S
from peanoclaw_gb300 import vtu


def _records(ps):
    return [vtu.patch_record_from_vector(ps.vector(p), ps.pos[p], ps.size[p], ps.n[p], ps.level[p],
                                         time=0.25, dt=0.01)
            for p in range(len(ps))]


def test_roundtrip_and_bounds(tmp_path):
    ps = S.uneven_patches(grid=3, sizes=(4, 8))
    recs = _records(ps)
    f = str(tmp_path / "out.vtu")
    vtu.write_vtu(f, recs)
    pts, conn, data = vtu.read_vtu(f)
    assert len(conn) == ps.cells()
    h = np.concatenate([r["fields"]["q0"].ravel() for r in recs])
    assert np.array_equal(data["q0"].view(np.int64), h.view(np.int64))
    b = np.concatenate([r["fields"]["pWG0"].ravel() for r in recs])
    assert np.array_equal(data["pWG0"], b)
    assert np.all(data["timeNew"] == 0.25 + 0.01)
    bd = vtu.cell_bounds(pts, conn)
    area = np.sum((bd[:, 1] - bd[:, 0]) * (bd[:, 3] - bd[:, 2]))
    assert abs(area - 1.0) < 1e-12
    # points are shared: a regular patch of n x n cells has (n+1)^2 points
    assert len(pts) < 4 * len(conn)


def test_compare_matches_cells_by_bounds(tmp_path):
    ps = S.radial_dam_break(npx=2, n=6)
    recs = _records(ps)
    fa, fb = str(tmp_path / "a.vtu"), str(tmp_path / "b.vtu")
    vtu.write_vtu(fa, recs)
    vtu.write_vtu(fb, list(reversed(recs)))      # same cells, other order
    a, b = vtu.read_vtu(fa), vtu.read_vtu(fb)
    assert vtu.compare_cells(a, b) == (0, 0.0)
    recs[1]["fields"]["q0"] = recs[1]["fields"]["q0"] + 1e-3
    vtu.write_vtu(fb, recs)
    missing, worst = vtu.compare_cells(a, vtu.read_vtu(fb))
    assert missing == 0 and abs(worst - 1e-3) < 1e-12
