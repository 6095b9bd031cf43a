"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  The product library never loads it.
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle

_lib = None


class PcoPatch(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("ghost", C.c_int32), ("nq", C.c_int32),
        ("np_wo", C.c_int32), ("np_w", C.c_int32), ("level", C.c_int32),
        ("is_leaf", C.c_int32), ("is_virtual", C.c_int32), ("pad_", C.c_int32),
        ("pos", C.c_double * 2), ("size", C.c_double * 2),
        ("time", C.c_double), ("dt", C.c_double), ("est_next", C.c_double),
        ("min_neighbor_time", C.c_double), ("max_neighbor_dt", C.c_double),
        ("restr_lower", C.c_double * 2), ("restr_upper", C.c_double * 2),
        ("u", C.POINTER(C.c_double)),
    ]


class PcoSweParams(C.Structure):
    _fields_ = [("g", C.c_double), ("cfl", C.c_double), ("dry_tol", C.c_double),
                ("dry_tol_update", C.c_double), ("s_min", C.c_double), ("dt_inf", C.c_double)]


class PcoGhostItem(C.Structure):
    _fields_ = [("kind", C.c_int32), ("src", C.c_int32), ("dst", C.c_int32),
                ("size", C.c_int32 * 2), ("src_offset", C.c_int32 * 2),
                ("dst_offset", C.c_int32 * 2)]


FLT_MAX = float(np.finfo(np.float32).max)


def swe_params(g=9.81, cfl=0.4, dry_tol=0.01, dry_tol_update=0.1, s_min=1e-5, dt_inf=FLT_MAX):
    return PcoSweParams(g, cfl, dry_tol, dry_tol_update, s_min, dt_inf)


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        P = C.POINTER(PcoPatch)
        D = C.POINTER(C.c_double)
        I2 = C.c_int * 2
        L.pco_patch_vector_size.argtypes = [P]
        L.pco_patch_vector_size.restype = C.c_int64
        for f in ("pco_idx_unew", "pco_idx_uold", "pco_idx_param_w"):
            getattr(L, f).argtypes = [P, C.c_int, C.c_int, C.c_int]
            getattr(L, f).restype = C.c_int64
        L.pco_idx_flux.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int]
        L.pco_idx_flux.restype = C.c_int64
        L.pco_fwave_edge.argtypes = [C.POINTER(PcoSweParams)] + [C.c_double] * 6 + [D]
        L.pco_copy_unew_to_uold.argtypes = [P]
        L.pco_swap_unew_uold.argtypes = [P]
        L.pco_swe_fill_boundary_layer.argtypes = [P, C.c_int, C.c_int]
        L.pco_swe_compute_net_updates.argtypes = [P, C.POINTER(PcoSweParams), D, D]
        L.pco_swe_compute_net_updates.restype = C.c_double
        L.pco_swe_update_unknowns.argtypes = [P, C.POINTER(PcoSweParams), D, C.c_double]
        L.pco_swe_solve_timestep.argtypes = [P, C.POINTER(PcoSweParams), C.c_double, D, D]
        L.pco_transfer_ghostlayer.argtypes = [I2, I2, I2, P, P]
        L.pco_interpolate.argtypes = [I2, I2, P, P, C.c_int, C.c_int, C.c_int, C.c_int]
        L.pco_restrict.argtypes = [P, P, C.c_int, C.c_int]
        L.pco_swe_post_process_restriction.argtypes = [P]
        L.pco_switch_to_leaf.argtypes = [P]
        L.pco_compute_fluxes.argtypes = [P, C.c_double]
        L.pco_apply_flux_correction.argtypes = [P, P, C.c_int, C.c_int]
        L.pco_region_map_to_patch.argtypes = [I2, I2, P, P, C.c_double, I2, I2]
        L.pco_regions_overlapped_by_ghostlayers.argtypes = [
            C.c_double * 2, C.c_double * 2, C.c_double * 2, C.c_double * 2, C.c_double * 2,
            I2, C.c_int * 8, C.c_int * 8]
        L.pco_regions_overlapped_by_ghostlayers.restype = C.c_int
        L.pco_overlap_area.argtypes = [C.c_double * 2] * 4
        L.pco_overlap_area.restype = C.c_double
        L.pco_grid_fill.argtypes = [C.POINTER(P), C.c_int, C.POINTER(PcoGhostItem), C.c_int,
                                    C.POINTER(C.c_uint8)]
        L.pco_grid_step.argtypes = [C.POINTER(P), C.c_int, C.POINTER(PcoGhostItem), C.c_int,
                                    C.POINTER(C.c_uint8), C.POINTER(C.c_int32), C.c_int,
                                    C.POINTER(PcoSweParams), D, D, C.c_int]
        L.pco32_grid_step.argtypes = [C.POINTER(P), C.POINTER(C.POINTER(C.c_float)), C.c_int,
                                      C.POINTER(PcoGhostItem), C.c_int, C.POINTER(C.c_uint8),
                                      C.POINTER(PcoSweParams), C.c_double, D, C.c_int]
        L.pco_grid_step_lts.restype = C.c_int
        L.pco_grid_step_lts.argtypes = [C.POINTER(P), C.c_int, C.POINTER(PcoGhostItem), C.c_int,
                                        C.POINTER(C.c_uint8), C.POINTER(PcoSweParams), C.c_double,
                                        C.c_double, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_int,
                                        D, C.c_int]
        _lib = L
    return _lib


class Patch:
    """A patch whose data vector lives in a numpy array (reference layout)."""

    def __init__(self, n, ghost=1, nq=3, np_wo=0, np_w=1, pos=(0.0, 0.0), size=(1.0, 1.0),
                 level=0, time=0.0, dt=0.0, is_leaf=True, is_virtual=False,
                 min_neighbor_time=0.0, max_neighbor_dt=0.0):
        nx, ny = (n, n) if np.isscalar(n) else n
        s = PcoPatch()
        s.nx, s.ny, s.ghost, s.nq, s.np_wo, s.np_w = nx, ny, ghost, nq, np_wo, np_w
        s.level, s.is_leaf, s.is_virtual = level, int(is_leaf), int(is_virtual)
        size = (size, size) if np.isscalar(size) else size
        s.pos[0], s.pos[1] = pos
        s.size[0], s.size[1] = size
        s.time, s.dt, s.est_next = time, dt, 0.0
        s.min_neighbor_time, s.max_neighbor_dt = min_neighbor_time, max_neighbor_dt
        s.restr_lower[0] = s.restr_lower[1] = np.finfo(np.float64).max
        s.restr_upper[0] = s.restr_upper[1] = -np.finfo(np.float64).max
        self.s = s
        self.u = np.zeros(lib().pco_patch_vector_size(C.byref(s)), dtype=np.float64)
        s.u = self.u.ctypes.data_as(C.POINTER(C.c_double))

    # layout views ------------------------------------------------------
    @property
    def nx(self):
        return self.s.nx

    @property
    def ny(self):
        return self.s.ny

    def _g(self):
        return self.s.ghost

    def unew(self):
        """(nq, nx, ny) view of uNew."""
        s = self.s
        return self.u[: s.nq * s.nx * s.ny].reshape(s.nq, s.nx, s.ny)

    def uold(self):
        """(nq, nx+2g, ny+2g) view of uOld with ghost layer; index +g."""
        s = self.s
        b = s.nq * s.nx * s.ny
        gx, gy = s.nx + 2 * s.ghost, s.ny + 2 * s.ghost
        return self.u[b: b + s.nq * gx * gy].reshape(s.nq, gx, gy)

    def param_w(self):
        s = self.s
        gx, gy = s.nx + 2 * s.ghost, s.ny + 2 * s.ghost
        b = s.nq * s.nx * s.ny + s.nq * gx * gy + s.np_wo * s.nx * s.ny
        return self.u[b: b + s.np_w * gx * gy].reshape(s.np_w, gx, gy)

    def flux(self):
        s = self.s
        gx, gy = s.nx + 2 * s.ghost, s.ny + 2 * s.ghost
        b = s.nq * s.nx * s.ny + s.nq * gx * gy + s.np_wo * s.nx * s.ny + s.np_w * gx * gy
        return self.u[b:]

    def ptr(self):
        return C.byref(self.s)

    def set_uold(self, x, y, q, v):
        self.u[lib().pco_idx_uold(self.ptr(), q, x, y)] = v

    def get_uold(self, x, y, q=0):
        return self.u[lib().pco_idx_uold(self.ptr(), q, x, y)]

    def set_unew(self, x, y, q, v):
        self.u[lib().pco_idx_unew(self.ptr(), q, x, y)] = v

    def get_unew(self, x, y, q=0):
        return self.u[lib().pco_idx_unew(self.ptr(), q, x, y)]


def ivec(v):
    return (C.c_int * 2)(*v)


def dvec(v):
    return (C.c_double * 2)(*v)


def fwave_edge(prm, hL, huL, bL, hR, huR, bR):
    out = (C.c_double * 5)()
    lib().pco_fwave_edge(C.byref(prm), hL, huL, bL, hR, huR, bR, out)
    return list(out)


def transfer_ghostlayer(size, src_off, dst_off, src, dst):
    lib().pco_transfer_ghostlayer(ivec(size), ivec(src_off), ivec(dst_off), src.ptr(), dst.ptr())


def interpolate(size, dst_off, src, dst, to_uold=True, to_current_time=False,
                use_time_unew_or_uold=True, swe=False):
    lib().pco_interpolate(ivec(size), ivec(dst_off), src.ptr(), dst.ptr(), int(to_uold),
                          int(to_current_time), int(use_time_unew_or_uold), int(swe))


def restrict(src, dst, only_overlapped=False, swe=False):
    lib().pco_restrict(src.ptr(), dst.ptr(), int(only_overlapped), int(swe))


def solve_timestep(p, prm, max_dt):
    dt = C.c_double()
    est = C.c_double()
    lib().pco_swe_solve_timestep(p.ptr(), C.byref(prm), max_dt, C.byref(dt), C.byref(est))
    return dt.value, est.value


def compute_net_updates(p, prm):
    A = (p.nx + 2) * (p.ny + 2)
    net = np.zeros(3 * A)
    smax = C.c_double()
    dt = lib().pco_swe_compute_net_updates(p.ptr(), C.byref(prm),
                                           net.ctypes.data_as(C.POINTER(C.c_double)),
                                           C.byref(smax))
    return dt, smax.value, net.reshape(3, p.nx + 2, p.ny + 2)


def ghost_items(items):
    """(N, 9) int32 array (or list of dicts) -> pco_ghost_item array."""
    if isinstance(items, np.ndarray):
        arr = np.ascontiguousarray(items, dtype=np.int32).reshape(-1, 9)
    else:
        arr = np.array([[it["kind"], it["src"], it["dst"], it["size"][0], it["size"][1],
                         it.get("src_offset", (0, 0))[0], it.get("src_offset", (0, 0))[1],
                         it["dst_offset"][0], it["dst_offset"][1]] for it in items],
                       dtype=np.int32).reshape(-1, 9)
    if len(arr) == 0:
        arr = np.zeros((1, 9), dtype=np.int32)
    arr = np.ascontiguousarray(arr)
    return arr.ctypes.data_as(C.POINTER(PcoGhostItem)), arr


def grid_step(patches, items, wall_mask, prm, max_dt, group=None, n_groups=1, n_threads=0):
    P = C.POINTER(PcoPatch)
    parr = (P * len(patches))(*[C.pointer(p.s) for p in patches])
    it, keep = ghost_items(items)
    wm = np.ascontiguousarray(wall_mask, dtype=np.uint8)
    grp = None if group is None else np.ascontiguousarray(group, dtype=np.int32)
    mdt = np.ascontiguousarray(np.broadcast_to(np.asarray(max_dt, dtype=np.float64), (n_groups,)))
    dto = np.zeros(n_groups)
    lib().pco_grid_step(parr, len(patches), it, len(keep) if len(items) else 0,
                        wm.ctypes.data_as(C.POINTER(C.c_uint8)),
                        None if grp is None else grp.ctypes.data_as(C.POINTER(C.c_int32)),
                        n_groups, C.byref(prm), mdt.ctypes.data_as(C.POINTER(C.c_double)),
                        dto.ctypes.data_as(C.POINTER(C.c_double)), n_threads)
    return dto


def grid_fill(patches, items, wall_mask):
    P = C.POINTER(PcoPatch)
    parr = (P * len(patches))(*[C.pointer(p.s) for p in patches])
    it, keep = ghost_items(items)
    wm = np.ascontiguousarray(wall_mask, dtype=np.uint8)
    lib().pco_grid_fill(parr, len(patches), it, len(keep) if len(items) else 0,
                        wm.ctypes.data_as(C.POINTER(C.c_uint8)))


def grid_step_lts(patches, items, wall_mask, prm, max_dt, t_end, virtual_time_items=None,
                  n_threads=0):
    """One local-time-stepping iteration; returns (number advanced, dt per
    patch).  virtual_time_items: (N, 2) (leaf, virtual ancestor) pairs whose
    intervals set the virtual patches' time intervals first."""
    P = C.POINTER(PcoPatch)
    parr = (P * len(patches))(*[C.pointer(p.s) for p in patches])
    it, keep = ghost_items(items)
    wm = np.ascontiguousarray(wall_mask, dtype=np.uint8)
    vt = np.zeros((0, 2), dtype=np.int32) if virtual_time_items is None else \
        np.ascontiguousarray(np.asarray(virtual_time_items, dtype=np.int32).reshape(-1, 2))
    vl, vv = np.ascontiguousarray(vt[:, 0]), np.ascontiguousarray(vt[:, 1])
    i32 = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))
    dto = np.zeros(len(patches))
    n = lib().pco_grid_step_lts(parr, len(patches), it, len(keep) if len(items) else 0,
                                wm.ctypes.data_as(C.POINTER(C.c_uint8)), C.byref(prm), float(max_dt),
                                float(t_end), i32(vl), i32(vv), len(vt),
                                dto.ctypes.data_as(C.POINTER(C.c_double)), n_threads)
    return n, dto



def grid_step_f32(patches, u32, items, wall_mask, prm, max_dt, n_threads=0):
    """FP32 twin of grid_step for one group (a timing baseline at the
    reference's float precision): u32[p] is patch p's data vector as float32
    in the layout of patches[p]; the patches' time intervals advance.
    Returns the dt taken."""
    P = C.POINTER(PcoPatch)
    F = C.POINTER(C.c_float)
    parr = (P * len(patches))(*[C.pointer(p.s) for p in patches])
    for a, p in zip(u32, patches):
        assert a.dtype == np.float32 and a.flags.c_contiguous and a.size == p.u.size
    uarr = (F * len(u32))(*[a.ctypes.data_as(F) for a in u32])
    it, keep = ghost_items(items)
    wm = np.ascontiguousarray(wall_mask, dtype=np.uint8)
    dto = C.c_double(0.0)
    lib().pco32_grid_step(parr, uarr, len(patches), it, len(keep) if len(items) else 0,
                          wm.ctypes.data_as(C.POINTER(C.c_uint8)), C.byref(prm), float(max_dt),
                          C.byref(dto), n_threads)
    return dto.value


def restrict_list(pats, restrict_items):
    """The batched restriction on oracle patches: every destination cleared
    (uNew and the uOld interior), the SWE restriction of every (src, dst) pair
    of the list in order, then postProcessRestriction of every destination
    (GridLevelTransfer.cpp:140-275)."""
    dsts = []
    for s, d in restrict_items:
        if int(d) not in dsts:
            dsts.append(int(d))
    for d in dsts:
        pats[d].unew()[:] = 0.0
        g = pats[d].s.ghost
        pats[d].uold()[:, g:-g, g:-g] = 0.0
    for s, d in restrict_items:
        restrict(pats[int(s)], pats[int(d)], only_overlapped=True, swe=True)
    for d in dsts:
        lib().pco_swe_post_process_restriction(pats[d].ptr())


def amr_step(pats, items, wall, leaf, flux_items, restrict_items, prm, max_dt, g_flux=1.0, flux=True,
             n_threads=0):
    """One synchronous step of an adaptive patch set on the oracle: ghost fill,
    sweep and update of the leaves (grid_step), then computeFluxes of every
    leaf and the flux-correction list (SolveTimestep.cpp:674-679), then the
    restriction list.  Returns the dt."""
    dt = grid_step(pats, items, wall, prm, max_dt, n_threads=n_threads)[0]
    if flux and len(flux_items):
        for p, lf in zip(pats, leaf):
            if lf:
                lib().pco_compute_fluxes(p.ptr(), g_flux)
        for s, d, dim, direction in flux_items:
            lib().pco_apply_flux_correction(pats[int(s)].ptr(), pats[int(d)].ptr(), int(dim), int(direction))
    restrict_list(pats, restrict_items)
    return dt
