"""ctypes binding of libpcg.so (include/pcg.h).

The library is built in-tree by peanoclaw_gb300.build; importing this module
never builds anything and never falls back to a CPU implementation: if the
shared library is missing the import of `lib()` raises.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libpcg.so")

PCG_OK = 0
PCG_E_INVALID = -1
PCG_E_NOMEM = -2
PCG_E_CUDA = -3
PCG_E_TIMEOUT = -4
PCG_E_STATE = -5
PCG_E_NUMERIC = -6
FORM_AUTO = 0
FORM_UNFUSED = 1
PCG_CRIT_DEPTH_GRADIENT = 0
PCG_CRIT_SURFACE_DIFFERENCE = 1
PCG_CRIT_SURFACE_GRADIENT = 2

PCG_PATCH_LEAF = 1
PCG_PATCH_VIRTUAL = 2
PCG_GHOST_COPY = 0
PCG_GHOST_INTERP = 1
PCG_MODE_PLAIN = 0
PCG_MODE_BATCHED = 1

FLT_MAX = float(np.finfo(np.float32).max)


class SweParams(C.Structure):
    _fields_ = [("g", C.c_double), ("cfl", C.c_double), ("dry_tol", C.c_double),
                ("dry_tol_update", C.c_double), ("s_min", C.c_double), ("dt_inf", C.c_double)]


class Config(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_patches", C.c_int32), ("max_groups", C.c_int32),
                ("reserved_", C.c_int32), ("slab_doubles", C.c_int64), ("params", SweParams)]


class PatchDesc(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("ghost", C.c_int32), ("nq", C.c_int32),
                ("np_wo", C.c_int32), ("np_w", C.c_int32), ("level", C.c_int32),
                ("flags", C.c_int32), ("pos", C.c_double * 2), ("size", C.c_double * 2)]


class PatchTime(C.Structure):
    _fields_ = [("time", C.c_double), ("dt", C.c_double), ("est_next", C.c_double),
                ("min_neighbor_time", C.c_double), ("max_neighbor_dt", C.c_double),
                ("restr_lower", C.c_double * 2), ("restr_upper", C.c_double * 2)]


class GhostItem(C.Structure):
    _fields_ = [("kind", C.c_int32), ("src", C.c_int32), ("dst", C.c_int32),
                ("size", C.c_int32 * 2), ("src_offset", C.c_int32 * 2),
                ("dst_offset", C.c_int32 * 2)]


class Schedule(C.Structure):
    _fields_ = [("kind", C.c_int32), ("variant", C.c_int32), ("chunk", C.c_int32),
                ("unfused", C.c_int32)]

    def as_tuple(self):
        return (self.kind, self.variant, self.chunk, self.unfused)


SCHED_TILES = 0
SCHED_STRIPS = 1
# values of the schedule's `unfused` field for strips
STRIPS_FUSED = 0       # the fused step where it applies
STRIPS_UNFUSED = 1     # separate launches
STRIPS_PIPELINED = 2   # one persistent kernel per step (pcg_pipeline.cu)
TS_GLOBAL = 0
TS_LOCAL = 1


# every entry point declared in include/pcg.h: name -> (restype, argtypes)
_CTX = C.c_void_p
_I2 = C.POINTER(C.c_int32)
_D = C.POINTER(C.c_double)
SIGNATURES = {
    "pcg_create": (C.c_int, [C.POINTER(Config), C.POINTER(_CTX)]),
    "pcg_destroy": (C.c_int, [_CTX]),
    "pcg_last_error": (C.c_char_p, []),
    "pcg_slab_info": (C.c_int, [_CTX, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "pcg_set_params": (C.c_int, [_CTX, C.POINTER(SweParams)]),
    "pcg_patch_alloc": (C.c_int, [_CTX, C.POINTER(PatchDesc), C.POINTER(C.c_int32)]),
    "pcg_patch_free": (C.c_int, [_CTX, C.c_int32]),
    "pcg_patch_vector_size": (C.c_int64, [C.POINTER(PatchDesc)]),
    "pcg_patch_upload": (C.c_int, [_CTX, C.c_int32, _D, C.c_int64]),
    "pcg_patch_download": (C.c_int, [_CTX, C.c_int32, _D, C.c_int64]),
    "pcg_patches_upload": (C.c_int, [_CTX, C.c_int32, _I2, _D]),
    "pcg_patches_download": (C.c_int, [_CTX, C.c_int32, _I2, _D]),
    "pcg_patch_set_desc_flags": (C.c_int, [_CTX, C.c_int32, C.c_int32]),
    "pcg_patch_set_time": (C.c_int, [_CTX, C.c_int32, C.POINTER(PatchTime)]),
    "pcg_patch_get_time": (C.c_int, [_CTX, C.c_int32, C.POINTER(PatchTime)]),
    "pcg_patch_set_boundary": (C.c_int, [_CTX, C.c_int32, C.c_uint32]),
    "pcg_patch_set_group": (C.c_int, [_CTX, C.c_int32, C.c_int32]),
    "pcg_copy_unew_to_uold": (C.c_int, [_CTX, C.c_int32]),
    "pcg_swap_unew_and_uold": (C.c_int, [_CTX, C.c_int32]),
    "pcg_fill_boundary_layer": (C.c_int, [_CTX, C.c_int32, C.c_int32, C.c_int32]),
    "pcg_solve_timestep": (C.c_int, [_CTX, C.c_int32, C.c_double, _D, _D]),
    "pcg_transfer_ghostlayer": (C.c_int, [_CTX, _I2, _I2, _I2, C.c_int32, C.c_int32]),
    "pcg_interpolate_solution": (C.c_int, [_CTX, _I2, _I2, C.c_int32, C.c_int32, C.c_int32,
                                           C.c_int32, C.c_int32, C.c_int32]),
    "pcg_restrict_solution": (C.c_int, [_CTX, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "pcg_post_process_restriction": (C.c_int, [_CTX, C.c_int32]),
    "pcg_compute_fluxes": (C.c_int, [_CTX, C.c_int32, C.c_double]),
    "pcg_apply_flux_correction": (C.c_int, [_CTX, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "pcg_set_ghost_items": (C.c_int, [_CTX, C.POINTER(GhostItem), C.c_int32]),
    "pcg_set_group_max_dt": (C.c_int, [_CTX, C.c_int32, C.c_double]),
    "pcg_set_group_end_time": (C.c_int, [_CTX, C.c_int32, C.c_double, C.c_double]),
    "pcg_set_time_stepping": (C.c_int, [_CTX, C.c_int32]),
    "pcg_set_virtual_time_items": (C.c_int, [_CTX, C.c_int32, _I2, _I2]),
    "pcg_get_group_times": (C.c_int, [_CTX, _D]),
    "pcg_set_restriction_items": (C.c_int, [_CTX, C.c_int32, _I2, _I2, C.c_int32]),
    "pcg_set_flux_correction_items": (C.c_int, [_CTX, C.c_int32, _I2, _I2, _I2, _I2, C.c_double]),
    "pcg_restrict_all": (C.c_int, [_CTX]),
    "pcg_clear_subgrid": (C.c_int, [_CTX, C.c_int32]),
    "pcg_gather_cells": (C.c_int, [_CTX, C.c_int32, _I2, _D, C.c_int64]),
    "pcg_patches_get_time": (C.c_int, [_CTX, C.c_int32, _I2, C.POINTER(PatchTime)]),
    "pcg_patches_set_restriction_bounds": (C.c_int, [_CTX, C.c_int32, _I2, _D, _D]),
    "pcg_patches_set_time": (C.c_int, [_CTX, C.c_int32, _I2, C.POINTER(PatchTime)]),
    "pcg_interpolate_solution_many": (C.c_int, [_CTX, C.c_int32, _I2, _I2, _I2, _I2, C.c_int32, C.c_int32,
                                                C.c_int32, C.c_int32]),
    "pcg_switch_to_leaf": (C.c_int, [_CTX, C.c_int32]),
    "pcg_amr_layout": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, _I2, _I2, _I2,
                                 C.POINTER(C.c_uint8), _I2, _I2, _I2, _I2, _I2, _I2, _D, _D, _I2]),
    "pcg_refinement_indicator": (C.c_int, [_CTX, C.c_int32, _I2, _D]),
    "pcg_refinement_criterion": (C.c_int, [_CTX, C.c_int32, _I2, C.c_int32, _D]),
    "pcg_step": (C.c_int, [_CTX, C.c_int32, _D]),
    "pcg_set_step_form": (C.c_int, [_CTX, C.c_int32]),
    "pcg_get_step_form": (C.c_int, [_CTX, C.c_int32, C.POINTER(C.c_int32)]),
    "pcg_get_step_launches": (C.c_int, [_CTX, C.POINTER(C.c_int32)]),
    "pcg_selftest_transfer_wait": (C.c_int, [_CTX]),
    "pcg_run": (C.c_int, [_CTX, C.c_int32, C.c_int32, _D]),
    "pcg_run_async": (C.c_int, [_CTX, C.c_int32, C.c_int32]),
    "pcg_run_wait": (C.c_int, [_CTX, _D]),
    "pcg_stats": (C.c_int, [_CTX, C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
    "pcg_synchronize": (C.c_int, [_CTX]),
    "pcg_set_schedule": (C.c_int, [_CTX, C.POINTER(Schedule)]),
    "pcg_get_schedule": (C.c_int, [_CTX, C.POINTER(Schedule)]),
    "pcg_autotune": (C.c_int, [_CTX, C.c_int32, C.POINTER(Schedule), _D, C.c_int32,
                               C.POINTER(C.c_int32)]),
    "pcg_profile_step": (C.c_int, [_CTX, _D]),
    "pcg_probe_fp64_peak": (C.c_int, [_CTX, _D]),
    "pcg_check_ieee_emulation": (C.c_int, [_CTX, C.c_int64, C.c_uint64, C.POINTER(C.c_int64)]),
    "pcg_solve_timestep_noalloc": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _D,
                                             C.POINTER(SweParams), C.c_double, _D, _D, C.c_void_p]),
}

_lib = None


class PcgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("pcg error %d: %s" % (code, msg))
        self.code = code


def lib():
    """Load libpcg.so; raises if the CUDA library has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libpcg.so not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc):
    if rc != PCG_OK:
        raise PcgError(rc, lib().pcg_last_error().decode())
    return rc


def i2(v):
    return (C.c_int32 * 2)(*[int(x) for x in v])


def dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def swe_params(g=9.81, cfl=0.4, dry_tol=0.01, dry_tol_update=0.1, s_min=1e-5, dt_inf=FLT_MAX):
    return SweParams(g, cfl, dry_tol, dry_tol_update, s_min, dt_inf)


def vector_size(n, ghost=1, nq=3, np_wo=0, np_w=1):
    nx, ny = (n, n) if np.isscalar(n) else n
    vn, vo = nx * ny, (nx + 2 * ghost) * (ny + 2 * ghost)
    return nq * vn + nq * vo + np_wo * vn + np_w * vo + 2 * nq * (nx + ny)


def items_array(items):
    """Ghost items as a contiguous (N, 9) int32 array in pcg_ghost_item layout."""
    if isinstance(items, np.ndarray):
        return np.ascontiguousarray(items, dtype=np.int32).reshape(-1, 9)
    rows = [[it["kind"], it["src"], it["dst"], it["size"][0], it["size"][1],
             it.get("src_offset", (0, 0))[0], it.get("src_offset", (0, 0))[1],
             it["dst_offset"][0], it["dst_offset"][1]] for it in items]
    return np.array(rows, dtype=np.int32).reshape(-1, 9)


class Context:
    """A device context: one HBM slab with every patch vector resident."""

    def __init__(self, slab_doubles, max_patches=1024, max_groups=1, params=None, device=0):
        cfg = Config()
        cfg.device = device
        cfg.max_patches = max_patches
        cfg.max_groups = max_groups
        cfg.slab_doubles = int(slab_doubles)
        cfg.params = params if params is not None else swe_params()
        self.max_groups = max_groups
        h = C.c_void_p()
        check(lib().pcg_create(C.byref(cfg), C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            lib().pcg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # patches --------------------------------------------------------------
    def alloc(self, n, ghost=1, nq=3, np_wo=0, np_w=1, pos=(0.0, 0.0), size=(1.0, 1.0),
              level=0, leaf=True, virtual=False):
        nx, ny = (n, n) if np.isscalar(n) else n
        size = (size, size) if np.isscalar(size) else size
        d = PatchDesc(nx, ny, ghost, nq, np_wo, np_w, level,
                      (PCG_PATCH_LEAF if leaf else 0) | (PCG_PATCH_VIRTUAL if virtual else 0),
                      (C.c_double * 2)(*pos), (C.c_double * 2)(*size))
        pid = C.c_int32()
        check(lib().pcg_patch_alloc(self.h, C.byref(d), C.byref(pid)))
        return pid.value

    def free(self, pid):
        check(lib().pcg_patch_free(self.h, pid))

    def upload(self, pid, vec):
        vec = np.ascontiguousarray(vec, dtype=np.float64)
        check(lib().pcg_patch_upload(self.h, pid, dptr(vec), vec.size))

    def download(self, pid, n):
        out = np.empty(n, dtype=np.float64)
        check(lib().pcg_patch_download(self.h, pid, dptr(out), n))
        return out

    def upload_many(self, ids, packed):
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        packed = np.ascontiguousarray(packed, dtype=np.float64)
        check(lib().pcg_patches_upload(self.h, len(ids), ids.ctypes.data_as(_I2), dptr(packed)))

    def download_many(self, ids, total):
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        out = np.empty(total, dtype=np.float64)
        check(lib().pcg_patches_download(self.h, len(ids), ids.ctypes.data_as(_I2), dptr(out)))
        return out

    def set_time(self, pid, time=0.0, dt=0.0, est_next=0.0, min_neighbor_time=0.0,
                 max_neighbor_dt=0.0, restr_lower=None, restr_upper=None):
        big = np.finfo(np.float64).max
        rl = restr_lower if restr_lower is not None else (big, big)
        ru = restr_upper if restr_upper is not None else (-big, -big)
        t = PatchTime(time, dt, est_next, min_neighbor_time, max_neighbor_dt,
                      (C.c_double * 2)(*rl), (C.c_double * 2)(*ru))
        check(lib().pcg_patch_set_time(self.h, pid, C.byref(t)))

    def get_time(self, pid):
        t = PatchTime()
        check(lib().pcg_patch_get_time(self.h, pid, C.byref(t)))
        return {"time": t.time, "dt": t.dt, "est_next": t.est_next,
                "min_neighbor_time": t.min_neighbor_time, "max_neighbor_dt": t.max_neighbor_dt}

    def set_boundary(self, pid, mask):
        check(lib().pcg_patch_set_boundary(self.h, pid, int(mask)))

    def set_group(self, pid, group):
        check(lib().pcg_patch_set_group(self.h, pid, int(group)))

    def set_flags(self, pid, leaf=True, virtual=False):
        check(lib().pcg_patch_set_desc_flags(
            self.h, pid, (PCG_PATCH_LEAF if leaf else 0) | (PCG_PATCH_VIRTUAL if virtual else 0)))

    def slab_info(self):
        f, t = C.c_int64(), C.c_int64()
        check(lib().pcg_slab_info(self.h, C.byref(f), C.byref(t)))
        return f.value, t.value

    # batched ----------------------------------------------------------------
    def set_ghost_items(self, items):
        """items: (N, 9) int32 array (kind, src, dst, size[2], src_offset[2],
        dst_offset[2]) or a list of dicts with those keys."""
        arr = items_array(items)
        ptr = arr.ctypes.data_as(C.POINTER(GhostItem)) if len(arr) else None
        check(lib().pcg_set_ghost_items(self.h, ptr, len(arr)))

    def set_restriction_items(self, src, dst, only_overlapped=True):
        src = np.ascontiguousarray(src, dtype=np.int32)
        dst = np.ascontiguousarray(dst, dtype=np.int32)
        check(lib().pcg_set_restriction_items(self.h, len(src), src.ctypes.data_as(_I2),
                                              dst.ctypes.data_as(_I2), int(only_overlapped)))

    def set_flux_correction_items(self, src, dst, dim, direction, g_flux=1.0):
        arrs = [np.ascontiguousarray(a, dtype=np.int32) for a in (src, dst, dim, direction)]
        check(lib().pcg_set_flux_correction_items(self.h, len(arrs[0]),
                                                  *[a.ctypes.data_as(_I2) for a in arrs], float(g_flux)))

    def restrict_all(self):
        check(lib().pcg_restrict_all(self.h))

    def set_group_max_dt(self, group, max_dt):
        check(lib().pcg_set_group_max_dt(self.h, group, float(max_dt)))

    def clear_subgrid(self, pid):
        check(lib().pcg_clear_subgrid(self.h, int(pid)))

    def gather_cells(self, ids, shapes):
        """uNew and the parameter interior of every patch in ids, back to back;
        shapes: per patch (nq + np_w) * nx * ny."""
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        out = np.empty(int(sum(shapes)))
        check(lib().pcg_gather_cells(self.h, len(ids), ids.ctypes.data_as(_I2), dptr(out), out.size))
        return out

    def times_of(self, ids):
        """(time, dt) of every patch in ids."""
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        arr = (PatchTime * max(1, len(ids)))()
        check(lib().pcg_patches_get_time(self.h, len(ids), ids.ctypes.data_as(_I2), arr))
        return np.array([[arr[k].time, arr[k].dt] for k in range(len(ids))]).reshape(-1, 2)

    def set_times_many(self, ids, time, dt, est_next):
        """Time, dt and estimated next dt of many patches in one call
        (pcg_patches_set_time; restriction bounds reset to empty)."""
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        big = np.finfo(np.float64).max
        arr = (PatchTime * max(1, len(ids)))()
        for k in range(len(ids)):
            arr[k] = PatchTime(float(time[k]), float(dt[k]), float(est_next[k]), 0.0, 0.0,
                               (C.c_double * 2)(big, big), (C.c_double * 2)(-big, -big))
        check(lib().pcg_patches_set_time(self.h, len(ids), ids.ctypes.data_as(_I2), arr))

    def interpolate_many(self, src, dst, size, dst_offset, to_uold, to_current, use_unew_uold, swe=True):
        """pcg_interpolate_solution_many: size and dst_offset are (n, 2)."""
        src = np.ascontiguousarray(src, dtype=np.int32)
        dst = np.ascontiguousarray(dst, dtype=np.int32)
        sz = np.ascontiguousarray(size, dtype=np.int32).reshape(-1, 2)
        of = np.ascontiguousarray(dst_offset, dtype=np.int32).reshape(-1, 2)
        check(lib().pcg_interpolate_solution_many(self.h, len(src), src.ctypes.data_as(_I2), dst.ctypes.data_as(_I2),
                                                  sz.ctypes.data_as(_I2), of.ctypes.data_as(_I2), int(to_uold),
                                                  int(to_current), int(use_unew_uold), int(swe)))

    def set_restriction_bounds(self, ids, lower, upper):
        """Restriction bounds of many patches (pcg_patches_set_restriction_bounds);
        lower and upper are (n, 2) arrays."""
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        lo = np.ascontiguousarray(lower, dtype=np.float64).reshape(-1, 2)
        up = np.ascontiguousarray(upper, dtype=np.float64).reshape(-1, 2)
        if len(lo) != len(ids) or len(up) != len(ids):
            raise ValueError("ids, lower and upper differ in length")
        check(lib().pcg_patches_set_restriction_bounds(self.h, len(ids), ids.ctypes.data_as(_I2), dptr(lo),
                                                       dptr(up)))

    def switch_to_leaf(self, pid):
        check(lib().pcg_switch_to_leaf(self.h, int(pid)))

    def refinement_indicator(self, ids, kind=None):
        """Refinement criterion of the listed patches (pcg_refinement_criterion;
        default: the BreakingDam depth gradient)."""
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        out = np.zeros(len(ids))
        if len(ids):
            k = PCG_CRIT_DEPTH_GRADIENT if kind is None else int(kind)
            check(lib().pcg_refinement_criterion(self.h, len(ids), ids.ctypes.data_as(C.POINTER(C.c_int32)),
                                                 k, dptr(out)))
        return out

    def set_group_end_time(self, group, time, t_end):
        """Device-side end time of a group (see pcg_set_group_end_time)."""
        check(lib().pcg_set_group_end_time(self.h, group, float(time), float(t_end)))

    def set_time_stepping(self, mode):
        """TS_GLOBAL (synchronous steps) or TS_LOCAL (local time stepping,
        batched form; see pcg_set_time_stepping)."""
        check(lib().pcg_set_time_stepping(self.h, int(mode)))

    def set_virtual_time_items(self, leaf, virt):
        """(leaf, virtual ancestor) pairs that set the virtual patches' time
        intervals in local time stepping (see pcg_set_virtual_time_items)."""
        leaf = np.ascontiguousarray(leaf, dtype=np.int32)
        virt = np.ascontiguousarray(virt, dtype=np.int32)
        if leaf.shape != virt.shape:
            raise ValueError("leaf and virt differ in length")
        check(lib().pcg_set_virtual_time_items(self.h, len(leaf), leaf.ctypes.data_as(_I2),
                                               virt.ctypes.data_as(_I2)))

    def group_times(self):
        out = np.zeros(self.max_groups)
        check(lib().pcg_get_group_times(self.h, dptr(out)))
        return out

    def step(self, mode=PCG_MODE_BATCHED):
        out = np.zeros(self.max_groups)
        check(lib().pcg_step(self.h, mode, dptr(out)))
        return out

    def set_step_form(self, form):
        """pcg_set_step_form: FORM_AUTO (fused where it applies) or FORM_UNFUSED."""
        check(lib().pcg_set_step_form(self.h, int(form)))

    def step_is_fused(self, mode=PCG_MODE_BATCHED):
        v = C.c_int32()
        check(lib().pcg_get_step_form(self.h, int(mode), C.byref(v)))
        return bool(v.value)

    def selftest_transfer_wait(self):
        """pcg_selftest_transfer_wait: the level transfer's bounded wait runs
        out on purpose and is reported; raises PcgError otherwise."""
        check(lib().pcg_selftest_transfer_wait(self.h))

    def step_launches(self):
        """Kernel launches of one captured batched step (pcg_get_step_launches)."""
        v = C.c_int32()
        check(lib().pcg_get_step_launches(self.h, C.byref(v)))
        return int(v.value)

    def run(self, steps, mode=PCG_MODE_BATCHED):
        hist = np.zeros(steps * self.max_groups)
        check(lib().pcg_run(self.h, steps, mode, dptr(hist)))
        return hist.reshape(steps, self.max_groups)

    def run_async(self, steps, mode=PCG_MODE_BATCHED):
        """pcg_run_async: enqueue `steps` steps and return; run_wait() ends the run."""
        check(lib().pcg_run_async(self.h, int(steps), mode))
        self._async_steps = int(steps)

    def run_wait(self):
        """pcg_run_wait: the dt history of the run started by run_async."""
        steps = self._async_steps
        hist = np.zeros(steps * self.max_groups)
        check(lib().pcg_run_wait(self.h, dptr(hist)))
        return hist.reshape(steps, self.max_groups)

    def stats(self):
        cu, ms = C.c_int64(), C.c_double()
        check(lib().pcg_stats(self.h, C.byref(cu), C.byref(ms)))
        return cu.value, ms.value

    def synchronize(self):
        check(lib().pcg_synchronize(self.h))

    def set_schedule(self, kind, variant=0, chunk=32, unfused=0):
        """Fix the batched sweep/update schedule (SCHED_TILES or SCHED_STRIPS;
        for strips, unfused = STRIPS_UNFUSED keeps the unfused step form and
        STRIPS_PIPELINED runs pcg_run in the pipelined form)."""
        s = Schedule(kind, variant, chunk, unfused)
        check(lib().pcg_set_schedule(self.h, C.byref(s)))

    def get_schedule(self):
        s = Schedule()
        check(lib().pcg_get_schedule(self.h, C.byref(s)))
        return s.as_tuple()

    def autotune(self, reps=2):
        """Time every candidate schedule over `reps` batched steps each (the
        simulation advances by those steps) and keep the fastest.  Returns
        [((kind, variant, chunk, unfused), mean ms per step), ...]."""
        cap = 64
        tried = (Schedule * cap)()
        ms = np.zeros(cap)
        n = C.c_int32()
        check(lib().pcg_autotune(self.h, int(reps), tried, dptr(ms), cap, C.byref(n)))
        return [(tried[k].as_tuple(), float(ms[k])) for k in range(min(n.value, cap))]

    def profile_step(self):
        """Device ms of (reset, ghost items, walls, sweep, update) of one batched
        step (fused and pipelined forms: see pcg_profile_step)."""
        ms = np.zeros(5)
        check(lib().pcg_profile_step(self.h, dptr(ms)))
        return ms

    def check_ieee_emulation(self, samples, seed=1):
        bad = C.c_int64()
        check(lib().pcg_check_ieee_emulation(self.h, int(samples), int(seed), C.byref(bad)))
        return bad.value

    def fp64_peak_tflops(self):
        v = C.c_double()
        check(lib().pcg_probe_fp64_peak(self.h, C.byref(v)))
        return v.value
