// drive_numerics.cpp -- test driver of the GPU Numerics plugin: plays the
// calls a Peano grid iteration makes on the numerics object, in the order of
// the reference's traversal, on subgrids whose data live on the device:
//   the compositor's ghost-layer transfers of every face pair
//   (GhostlayerCompositorFunctors.cpp:59-69, through the virtual
//   transferGhostlayer / interpolateSolution), then per subgrid
//   SolveTimestep::enterCell (SolveTimestep.cpp:591-700):
//   DefaultTransfer::copyUNewToUOld, the domain boundary layers in the order
//   of fillBoundaryLayers (SolveTimestep.cpp:87-142), solveTimestep with the
//   global timestep bound, getDemandedMeshWidth.
// Everything goes through a peanoclaw::Numerics reference.
#include <cstdint>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "GpuSWEKernel.h"

namespace {
std::string g_error;
}

extern "C" const char *shim_last_error() { return g_error.c_str(); }

// n subgrids already allocated in `ctx` (ids, geometry, wall masks: bit
// 2 dim + upper), items[9 k ..] the ghost face pairs (kind, src, dst, size,
// src offset, dst offset as indices into the subgrid arrays), `steps` grid
// iterations with global timestep bound max_dt.  Outputs per iteration and
// subgrid: dt taken, CFL estimate, demanded mesh width (x).
extern "C" int shim_drive_iterations(pcg_context *ctx, int32_t n, const int32_t *ids, const double *pos,
                                     const double *size, const int32_t *subdivision, const uint8_t *walls,
                                     int32_t n_items, const int32_t *items, int32_t steps, double max_dt,
                                     double *dt_out, double *est_out, double *width_out) {
  try {
    using namespace peanoclaw;
    native::GpuRefinementCriterion crit;
    crit.kind = PCG_CRIT_DEPTH_GRADIENT;
    crit.threshold = 0.1;
    crit.minimalMeshWidth = 1.0 / 243.0;
    crit.maximalMeshWidth = 1.0 / 27.0;
    native::GpuSWEKernel kernel(ctx, crit);
    Numerics &numerics = kernel;
    std::vector<records::CellDescription> cells(n);
    for (int p = 0; p < n; p++) {
      records::CellDescription &cd = cells[p];
      cd.subdivisionFactor[0] = cd.subdivisionFactor[1] = subdivision[p];
      cd.position[0] = pos[2 * p];
      cd.position[1] = pos[2 * p + 1];
      cd.size[0] = size[2 * p];
      cd.size[1] = size[2 * p + 1];
      cd.uIndex = ids[p];
    }
    interSubgridCommunication::DefaultTransfer transfer;
    for (int s = 0; s < steps; s++) {
      for (int k = 0; k < n_items; k++) {
        const int32_t *it = items + 9 * k;
        Patch source(cells[it[1]]), destination(cells[it[2]]);
        tarch::la::Vector<DIMENSIONS, int> sz, so, dof;
        sz[0] = it[3]; sz[1] = it[4];
        so[0] = it[5]; so[1] = it[6];
        dof[0] = it[7]; dof[1] = it[8];
        if (it[0] == PCG_GHOST_COPY) numerics.transferGhostlayer(sz, so, dof, source, destination);
        else numerics.interpolateSolution(sz, dof, source, destination, true, false, true);
      }
      for (int p = 0; p < n; p++) {
        Patch subgrid(cells[p]);
        transfer.copyUNewToUOld(subgrid);
        tarch::la::Vector<DIMENSIONS_TIMES_TWO, bool> flags(false);
        if (walls[p] & 1) { numerics.fillBoundaryLayer(subgrid, 0, false); flags[0] = true; }
        if (walls[p] & 8) { numerics.fillBoundaryLayer(subgrid, 1, true); flags[3] = true; }
        if (walls[p] & 2) { numerics.fillBoundaryLayer(subgrid, 0, true); flags[1] = true; }
        if (walls[p] & 4) { numerics.fillBoundaryLayer(subgrid, 1, false); flags[2] = true; }
        numerics.solveTimestep(subgrid, max_dt, false, flags);
        subgrid.setDemandedMeshWidth(numerics.getDemandedMeshWidth(subgrid, false));
        dt_out[(int64_t)s * n + p] = subgrid.getTimeIntervals().getTimestepSize();
        est_out[(int64_t)s * n + p] = subgrid.getTimeIntervals().getEstimatedNextTimestepSize();
        width_out[(int64_t)s * n + p] = subgrid.getDemandedMeshWidth()[0];
      }
    }
    return 0;
  } catch (const std::exception &e) {
    g_error = e.what();
    return 1;
  }
}
