"""Host-side mirror of peanoclaw::Numerics for the GB300 SWE kernel.

`SWEKernel` keeps the reference's method names, argument meaning and
defaults (src/peanoclaw/Numerics.h:30-204, src/peanoclaw/native/SWEKernel.h);
each method forwards to one entry point of libpcg.so.  Patch data never
leaves the device; `Patch` is a handle (slab id + geometry), the analogue of
the transient peanoclaw::Patch views the traversal creates per event.
"""
import numpy as np

from . import pcg as _pcg


class Patch:
    """Handle of one device-resident subgrid."""

    def __init__(self, ctx, subdivision, position, size, level=0, ghost=1, unknowns=3,
                 params_without_ghost=0, params_with_ghost=1, leaf=True, virtual=False):
        self.ctx = ctx
        self.subdivision = (subdivision, subdivision) if np.isscalar(subdivision) else tuple(subdivision)
        self.position = tuple(position)
        self.size = (size, size) if np.isscalar(size) else tuple(size)
        self.level = level
        self.ghost = ghost
        self.unknowns = unknowns
        self.id = ctx.alloc(self.subdivision, ghost, unknowns, params_without_ghost,
                            params_with_ghost, self.position, self.size, level, leaf, virtual)
        self.vector_size = _pcg.vector_size(self.subdivision, ghost, unknowns,
                                            params_without_ghost, params_with_ghost)

    def upload(self, vec):
        self.ctx.upload(self.id, vec)

    def download(self):
        return self.ctx.download(self.id, self.vector_size)

    def set_time_intervals(self, **kw):
        self.ctx.set_time(self.id, **kw)

    def get_time_intervals(self):
        return self.ctx.get_time(self.id)


class SWEKernel:
    """peanoclaw::native::SWEKernel on the GPU (src/peanoclaw/native/SWEKernel.h:32-167)."""

    def __init__(self, ctx):
        self.ctx = ctx

    # sizes (SWEKernel.h:124-133)
    def getNumberOfUnknownsPerCell(self):
        return 3

    def getNumberOfParameterFieldsWithoutGhostlayer(self):
        return 0

    def getNumberOfParameterFieldsWithGhostlayer(self):
        return 1

    def getGhostlayerWidth(self):
        return 1

    # hot path
    def solveTimestep(self, subgrid, maximumTimestepSize, useDimensionalSplitting=False,
                      domainBoundaryFlags=None):
        """Returns (dt used, estimated next timestep size)."""
        import ctypes as C
        dt = C.c_double()
        est = C.c_double()
        _pcg.check(_pcg.lib().pcg_solve_timestep(self.ctx.h, subgrid.id, float(maximumTimestepSize),
                                                 C.byref(dt), C.byref(est)))
        return dt.value, est.value

    def fillBoundaryLayer(self, subgrid, dimension, setUpper):
        _pcg.check(_pcg.lib().pcg_fill_boundary_layer(self.ctx.h, subgrid.id, int(dimension),
                                                      int(bool(setUpper))))

    def copyUNewToUOld(self, subgrid):
        """DefaultTransfer::copyUNewToUOld, done by SolveTimestep before the solve."""
        _pcg.check(_pcg.lib().pcg_copy_unew_to_uold(self.ctx.h, subgrid.id))

    def transferGhostlayer(self, size, sourceOffset, destinationOffset, source, destination):
        _pcg.check(_pcg.lib().pcg_transfer_ghostlayer(self.ctx.h, _pcg.i2(size), _pcg.i2(sourceOffset),
                                                      _pcg.i2(destinationOffset), source.id,
                                                      destination.id))

    def interpolateSolution(self, destinationSize, destinationOffset, source, destination,
                            interpolateToUOld=True, interpolateToCurrentTime=True,
                            useTimeUNewOrTimeUOld=True):
        """SWEKernel::interpolateSolution: interpolation of the absolute surface h+b."""
        _pcg.check(_pcg.lib().pcg_interpolate_solution(
            self.ctx.h, _pcg.i2(destinationSize), _pcg.i2(destinationOffset), source.id,
            destination.id, int(interpolateToUOld), int(interpolateToCurrentTime),
            int(useTimeUNewOrTimeUOld), 1))

    def restrictSolution(self, source, destination, restrictOnlyOverlappedRegions):
        _pcg.check(_pcg.lib().pcg_restrict_solution(self.ctx.h, source.id, destination.id,
                                                    int(restrictOnlyOverlappedRegions), 1))

    def postProcessRestriction(self, destination, restrictOnlyOverlappedRegions=False):
        _pcg.check(_pcg.lib().pcg_post_process_restriction(self.ctx.h, destination.id))

    def computeFluxes(self, subgrid, g_flux=1.0):
        _pcg.check(_pcg.lib().pcg_compute_fluxes(self.ctx.h, subgrid.id, float(g_flux)))

    def applyFluxCorrection(self, sourceSubgrid, destinationSubgrid, dimension, direction):
        _pcg.check(_pcg.lib().pcg_apply_flux_correction(self.ctx.h, sourceSubgrid.id,
                                                        destinationSubgrid.id, int(dimension),
                                                        int(direction)))


class DefaultNumerics(SWEKernel):
    """The generic Numerics (NumericsTestStump-like): interpolation and
    restriction without the SWE h+b wrapping, any number of unknowns."""

    def interpolateSolution(self, destinationSize, destinationOffset, source, destination,
                            interpolateToUOld=True, interpolateToCurrentTime=True,
                            useTimeUNewOrTimeUOld=True):
        _pcg.check(_pcg.lib().pcg_interpolate_solution(
            self.ctx.h, _pcg.i2(destinationSize), _pcg.i2(destinationOffset), source.id,
            destination.id, int(interpolateToUOld), int(interpolateToCurrentTime),
            int(useTimeUNewOrTimeUOld), 0))

    def restrictSolution(self, source, destination, restrictOnlyOverlappedRegions):
        _pcg.check(_pcg.lib().pcg_restrict_solution(self.ctx.h, source.id, destination.id,
                                                    int(restrictOnlyOverlappedRegions), 0))
