"""PyClaw-style driver on the GPU: the `Peano` class of PeanoClaw's Python
package (src/python/peanoclaw/peano.py:17-200) backed by a pcg.Context.

The reference's `Peano` loads libpeano-claw-2d.so and calls
pyclaw_peano_new / evolveToTime / gatherSolution / destroy
(src/peanoclaw/pyclaw/pyclawBindings.cpp:108-340), which call back into
Python per subgrid with numpy views of the subgrid's arrays
(PyClawState.cpp:13-58: q = uNew (nq, nx, ny), qbc = uOld with ghost layer
(nq, nx+2g, ny+2g), aux = parameters without ghost layer).  This class keeps
that constructor, those methods and the callback conventions, for shallow
water problems solved by the GPU SWE kernel:

- the grid is the uniform spacetree level whose cell width is
  `initial_minimal_mesh_width`, each cell a subgrid of
  `solution.state.grid.dimensions[d].num_cells` cells;
- the initialization callback fills q (h, hu, hv) and, when the problem has
  one aux field, the bathymetry b of every subgrid (called with the
  reference's arguments; its return value, the demanded mesh width, is
  accepted and ignored: the grid stays uniform);
- the solver callback is not called: the GPU f-wave kernel advances all
  subgrids (synchronous global time stepping); domain boundaries are
  reflecting walls (the SWE kernel's fillBoundaryLayer), the boundary
  condition callback is not called;
- evolve_to_time runs batched steps until the end time (device-side end
  time, so the last step lands on it);
- gather_solution calls the addPatchToSolution callback per subgrid with
  views of the final data and the subgrid's new time.
"""
import numpy as np

from . import pcg as P
from .scenarios import PatchSet, _build_grid_items, remap_items


def _cb(obj, getter):
    """A reference callback object (with get_*_callback) or a plain callable."""
    if obj is None:
        return None
    f = getattr(obj, getter, None)
    return f() if f is not None else obj


class Peano:
    def __init__(self, solution, initial_minimal_mesh_width, ghostlayer_width, dt_initial,
                 initialization_callback, solver_callback=None, refinement_criterion_callback=None,
                 boundary_condition_callback=None, interpolation_callback=None,
                 restriction_callback=None, flux_correction_callback=None, internal_settings=None,
                 params=None, device=0):
        dims = solution.state.grid.dimensions
        if len(dims) != 2:
            raise ValueError("the GPU SWE kernel is two-dimensional")
        if ghostlayer_width != 1:
            raise ValueError("the GPU SWE kernel uses ghost layer width 1")
        nq = solution.state.num_eqn
        naux = solution.state.num_aux
        if nq != 3 or naux not in (0, 1):
            raise ValueError("shallow water: 3 unknowns and at most one aux field (bathymetry)")
        self.solution = solution
        self.internal_settings = internal_settings
        n = (dims[0].num_cells, dims[1].num_cells)
        if n[0] != n[1]:
            raise ValueError("square subgrids only")
        n = n[0]
        lo = (dims[0].lower, dims[1].lower)
        ext = (dims[0].upper - dims[0].lower, dims[1].upper - dims[1].lower)
        npx = [max(1, int(round(ext[d] / initial_minimal_mesh_width))) for d in (0, 1)]
        L = (ext[0] / npx[0], ext[1] / npx[1])
        self.n, self.naux = n, naux
        ps = PatchSet()
        grid = np.zeros((npx[0], npx[1]), dtype=np.int64)
        for i in range(npx[0]):
            for j in range(npx[1]):
                grid[i, j] = len(ps.n)
                ps.n.append(n)
                ps.pos.append((lo[0] + i * L[0], lo[1] + j * L[1]))
                ps.size.append(L)
                ps.level.append(0)
                m = 0
                if i == 0: m |= 1
                if i == npx[0] - 1: m |= 2
                if j == 0: m |= 4
                if j == npx[1] - 1: m |= 8
                ps.wall.append(m)
        ps.finalize_layout()
        init = _cb(initialization_callback, "get_initialization_callback")
        B = np.zeros((npx[0] * n, npx[1] * n))
        for i in range(npx[0]):
            for j in range(npx[1]):
                p = grid[i, j]
                unew, uold, b = ps.views(p)
                aux = np.zeros((naux, n, n))
                init(unew, uold, aux, n, n, 0, nq, naux, L[0], L[1], 0.0, ps.pos[p][0], ps.pos[p][1],
                     0.0, False)
                if naux:
                    B[i * n:(i + 1) * n, j * n:(j + 1) * n] = aux[0]
        if naux:
            # ghost bathymetry from the neighbouring subgrids; at the domain
            # boundary the boundary cell's value (mirror of a reflecting wall)
            Bg = np.pad(B, 1, mode="edge")
            for i in range(npx[0]):
                for j in range(npx[1]):
                    _, _, b = ps.views(grid[i, j])
                    b[:] = Bg[i * n:i * n + n + 2, j * n:j * n + n + 2]
        ps.items = _build_grid_items(ps, grid, npx[0], npx[1])
        self.ps = ps
        prm = params if params is not None else P.swe_params(g=9.81, cfl=0.5)
        self.ctx = P.Context(slab_doubles=int(ps.packed.size * 1.2) + 65536, max_patches=len(ps) + 8,
                             max_groups=1, params=prm, device=device)
        self.ids = []
        for p in range(len(ps)):
            pid = self.ctx.alloc(n, pos=ps.pos[p], size=ps.size[p])
            self.ctx.set_boundary(pid, ps.wall[p])
            self.ctx.set_time(pid, time=0.0, dt=0.0, est_next=dt_initial)
            self.ids.append(pid)
        self.ctx.upload_many(self.ids, ps.packed)
        self.ctx.set_ghost_items(remap_items(ps.items, self.ids))
        self.ctx.set_group_max_dt(0, np.inf)
        self.time = 0.0
        self.rank = 0
        self.add_to_solution = None
        if hasattr(solution, "peano"):
            solution.peano = self

    # -- reference methods (peano.py)
    def evolve_to_time(self, tend):
        """Advance every subgrid to `tend` (batched GPU steps)."""
        self.ctx.set_group_end_time(0, self.time, tend)
        t = self.time
        while t < tend:
            self.ctx.run(16, P.PCG_MODE_BATCHED)
            t_new = float(self.ctx.group_times()[0])
            if not t_new > t:
                raise RuntimeError("no progress towards t = %g (time %g)" % (tend, t_new))
            t = t_new
        self.time = t

    def gather_solution(self, add_patch_to_solution_callback=None):
        """Call the addPatchToSolution callback with every subgrid's q, qbc,
        ghost width, size, position and new time."""
        cb = _cb(add_patch_to_solution_callback or self.add_to_solution,
                 "get_add_to_solution_callback")
        data = self.ctx.download_many(self.ids, int(self.ps.packed.size))
        ps = self.ps
        for p in range(len(ps)):
            o = ps.offsets[p]
            vec = data[o:o + ps.vec_len(p)]
            n = ps.n[p]
            q = vec[:3 * n * n].reshape(3, n, n)
            qbc = vec[3 * n * n:3 * n * n + 3 * (n + 2) ** 2].reshape(3, n + 2, n + 2)
            t = self.ctx.get_time(self.ids[p])
            if cb is not None:
                cb(q, qbc, 1, ps.size[p][0], ps.size[p][1], 0.0, ps.pos[p][0], ps.pos[p][1], 0.0,
                   t["time"] + t["dt"])
        return data

    def teardown(self):
        self.ctx.close()

    def getRank(self):
        return self.rank

    def run_tests(self):
        return None
