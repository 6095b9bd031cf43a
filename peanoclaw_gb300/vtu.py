"""VTU output of the leaf patches, fed from the device buffers.

Writes what VTUSubgridPlotter writes for every subcell of every leaf patch
(src/peanoclaw/grid/plotter/VTUSubgridPlotter.cpp:118-186): one quadrilateral
per subcell with the unknowns of uNew as cell data "q0".."q{nq-1}", the
parameters with ghost layer as "pWG0".., and the meta information
"SubdivisionFactor", "GhostlayerWidth", "timeOld", "timeNew" (plus "level").
Points are shared between cells (the plotter's vertex-to-index map).  The
file is a VTK XML UnstructuredGrid with binary (base64, UInt64 header) inline
arrays.  The cell data come from the device in one gather
(pcg_gather_cells) and one copy.

`read_vtu` reads such a file back and `compare_cells` matches the cells of
two outputs by their bounds and reports the largest difference of a field,
which is what testscenarios/tools/compareResult.py:49-107 does with q0.
"""
import base64
import struct
import xml.etree.ElementTree as ET

import numpy as np

VTK_QUAD = 9


def _b64(arr):
    raw = np.ascontiguousarray(arr).tobytes()
    return base64.b64encode(struct.pack("<Q", len(raw)) + raw).decode("ascii")


def _vtk_type(dtype):
    return {np.dtype(np.float64): "Float64", np.dtype(np.int64): "Int64",
            np.dtype(np.uint8): "UInt8", np.dtype(np.int32): "Int32"}[np.dtype(dtype)]


def patch_records_from_context(ctx, ids, geometry, nq=3, np_w=1, ghost=1):
    """Records of the patches `ids` of a pcg.Context; geometry[k] =
    (pos, size, (nx, ny), level).  One device gather for all cell data."""
    shapes = [(nq + np_w) * g[2][0] * g[2][1] for g in geometry]
    flat = ctx.gather_cells(ids, shapes)
    times = ctx.times_of(ids)
    recs, o = [], 0
    for k, (pos, size, (nx, ny), level) in enumerate(geometry):
        nc = nx * ny
        blk = flat[o:o + (nq + np_w) * nc].reshape(nq + np_w, nx, ny)
        o += (nq + np_w) * nc
        fields = {"q%d" % q: blk[q] for q in range(nq)}
        fields.update({"pWG%d" % q: blk[nq + q] for q in range(np_w)})
        recs.append({"pos": pos, "size": size, "n": (nx, ny), "level": level, "ghost": ghost,
                     "time": float(times[k, 0]), "dt": float(times[k, 1]), "fields": fields})
    return recs


def patch_record_from_vector(vec, pos, size, n, level=0, time=0.0, dt=0.0, nq=3, np_w=1, ghost=1):
    """Record of one patch from its data vector in the reference layout."""
    nx, ny = (n, n) if np.isscalar(n) else n
    nc = nx * ny
    go = (nx + 2 * ghost) * (ny + 2 * ghost)
    fields = {"q%d" % q: vec[q * nc:(q + 1) * nc].reshape(nx, ny) for q in range(nq)}
    base = nq * nc + nq * go
    for q in range(np_w):
        full = vec[base + q * go: base + (q + 1) * go].reshape(nx + 2 * ghost, ny + 2 * ghost)
        fields["pWG%d" % q] = full[ghost:ghost + nx, ghost:ghost + ny]
    return {"pos": pos, "size": size, "n": (nx, ny), "level": level, "ghost": ghost,
            "time": time, "dt": dt, "fields": fields}


def write_vtu(path, records):
    """Write the subcells of the given patch records as one VTU file."""
    pts, cells, data = [], [], {}
    names = list(records[0]["fields"]) if records else []
    meta = {"SubdivisionFactor": [], "GhostlayerWidth": [], "timeOld": [], "timeNew": [], "level": []}
    for r in records:
        nx, ny = r["n"]
        hx, hy = r["size"][0] / nx, r["size"][1] / ny
        xs = r["pos"][0] + np.arange(nx + 1) * hx
        ys = r["pos"][1] + np.arange(ny + 1) * hy
        X, Y = np.meshgrid(xs, ys, indexing="ij")
        base = sum(len(p) for p in pts)
        pts.append(np.stack([X.ravel(), Y.ravel()], axis=1))
        ix, iy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
        v00 = base + ix * (ny + 1) + iy
        quad = np.stack([v00, v00 + (ny + 1), v00 + (ny + 1) + 1, v00 + 1], axis=-1).reshape(-1, 4)
        cells.append(quad)
        for name in names:
            data.setdefault(name, []).append(np.asarray(r["fields"][name], dtype=np.float64).ravel())
        nc = nx * ny
        meta["SubdivisionFactor"].append(np.full(nc, float(nx)))
        meta["GhostlayerWidth"].append(np.full(nc, float(r["ghost"])))
        meta["timeOld"].append(np.full(nc, r["time"]))
        meta["timeNew"].append(np.full(nc, r["time"] + r["dt"]))
        meta["level"].append(np.full(nc, float(r["level"])))
    P = np.concatenate(pts) if pts else np.zeros((0, 2))
    Cn = np.concatenate(cells) if cells else np.zeros((0, 4), dtype=np.int64)
    # shared points: the plotter's vertex-to-index map (exact coordinates)
    uniq, inv = np.unique(P, axis=0, return_inverse=True)
    Cn = inv.reshape(-1)[Cn].astype(np.int64)
    P3 = np.zeros((len(uniq), 3))
    P3[:, :2] = uniq
    nc = len(Cn)
    root = ET.Element("VTKFile", type="UnstructuredGrid", version="1.0", byte_order="LittleEndian",
                      header_type="UInt64")
    ug = ET.SubElement(root, "UnstructuredGrid")
    piece = ET.SubElement(ug, "Piece", NumberOfPoints=str(len(P3)), NumberOfCells=str(nc))

    def arr(parent, name, a, ncomp=1):
        a = np.ascontiguousarray(a)
        e = ET.SubElement(parent, "DataArray", type=_vtk_type(a.dtype), Name=name,
                          NumberOfComponents=str(ncomp), format="binary")
        e.text = _b64(a)

    arr(ET.SubElement(piece, "Points"), "Points", P3, 3)
    ce = ET.SubElement(piece, "Cells")
    arr(ce, "connectivity", Cn.ravel())
    arr(ce, "offsets", np.arange(4, 4 * nc + 1, 4, dtype=np.int64))
    arr(ce, "types", np.full(nc, VTK_QUAD, dtype=np.uint8))
    cd = ET.SubElement(piece, "CellData", Scalars=names[0] if names else "")
    for name in names:
        arr(cd, name, np.concatenate(data[name]))
    for name, parts in meta.items():
        arr(cd, name, np.concatenate(parts) if parts else np.zeros(0))
    ET.ElementTree(root).write(path, xml_declaration=True, encoding="utf-8")


def _decode(e, header="UInt64"):
    raw = base64.b64decode(e.text.strip())
    hs = 8 if header == "UInt64" else 4
    n = struct.unpack("<Q" if hs == 8 else "<I", raw[:hs])[0]
    dt = {"Float64": np.float64, "Int64": np.int64, "UInt8": np.uint8, "Int32": np.int32}[e.get("type")]
    return np.frombuffer(raw[hs:hs + n], dtype=dt)


def read_vtu(path):
    """(points (N,3), connectivity (M,4), cell data dict) of a file of write_vtu."""
    root = ET.parse(path).getroot()
    header = root.get("header_type", "UInt32")
    piece = root.find("UnstructuredGrid/Piece")
    pts = _decode(piece.find("Points/DataArray"), header).reshape(-1, 3)
    conn = None
    for e in piece.find("Cells"):
        if e.get("Name") == "connectivity":
            conn = _decode(e, header).reshape(-1, 4)
    data = {e.get("Name"): _decode(e, header) for e in piece.find("CellData")}
    return pts, conn, data


def cell_bounds(pts, conn):
    """(M, 4) xmin, xmax, ymin, ymax of every cell."""
    xy = pts[:, :2][conn]
    return np.stack([xy[..., 0].min(1), xy[..., 0].max(1), xy[..., 1].min(1), xy[..., 1].max(1)], axis=1)


def compare_cells(a, b, field="q0", accuracy=1e-8):
    """Match the cells of two read_vtu results by bounds (within `accuracy`)
    and return (number of cells of `a` without a match in `b`, largest
    |a.field - b.field| over the matched cells)."""
    pa, ca, da = a
    pb, cb, db = b
    ba, bb = cell_bounds(pa, ca), cell_bounds(pb, cb)
    key = lambda bd: tuple(np.round(bd / accuracy).astype(np.int64))
    index = {key(bd): k for k, bd in enumerate(bb)}
    missing, worst = 0, 0.0
    for k, bd in enumerate(ba):
        j = index.get(key(bd))
        if j is None:
            missing += 1
            continue
        worst = max(worst, abs(float(da[field][k]) - float(db[field][j])))
    return missing, worst
