// GpuSWEKernel.cpp -- implementation of the GB300 Numerics plugin and of the
// DefaultTransfer operations for device subgrids.
#include "GpuSWEKernel.h"

#include <stdexcept>
#include <string>

namespace peanoclaw {
namespace native {

namespace {

pcg_context *g_context = nullptr;

void check(int rc, const char *what) {
  if (rc != PCG_OK) throw std::runtime_error(std::string(what) + ": " + pcg_last_error());
}

int32_t deviceId(const Patch &patch) {
  if (patch.getUIndex() < 0) throw std::runtime_error("subgrid has no device patch (uIndex < 0)");
  return patch.getUIndex();
}

// The subgrid's time interval (CellDescription) to its device record.
void pushTime(pcg_context *c, Patch &patch) {
  peanoclaw::records::CellDescription &cd = patch.getCellDescription();
  pcg_patch_time t;
  t.time = cd.time;
  t.dt = cd.timestepSize;
  t.est_next = cd.estimatedNextTimestepSize;
  t.min_neighbor_time = cd.minimalNeighborTime;
  t.max_neighbor_dt = cd.maximalNeighborTimestep;
  for (int d = 0; d < 2; d++) {
    t.restr_lower[d] = cd.lowerNeighboringGhostlayerBounds[d];
    t.restr_upper[d] = cd.upperNeighboringGhostlayerBounds[d];
  }
  check(pcg_patch_set_time(c, deviceId(patch), &t), "pcg_patch_set_time");
}

// The device record back to the subgrid's time interval.
void pullTime(pcg_context *c, Patch &patch) {
  pcg_patch_time t;
  check(pcg_patch_get_time(c, deviceId(patch), &t), "pcg_patch_get_time");
  peanoclaw::records::CellDescription &cd = patch.getCellDescription();
  cd.time = t.time;
  cd.timestepSize = t.dt;
  cd.estimatedNextTimestepSize = t.est_next;
}

int32_t flagsOf(const peanoclaw::records::CellDescription &cd) {
  return (cd.isLeaf ? PCG_PATCH_LEAF : 0) | (cd.isVirtual ? PCG_PATCH_VIRTUAL : 0);
}

// The generic strategies of the Numerics base class (NumericsFactory passes
// DefaultInterpolation, DefaultRestriction and DefaultFluxCorrection,
// NumericsFactory.cpp:28-51): the same operations without the SWE h + b
// wrapping.
class GpuInterpolation : public peanoclaw::interSubgridCommunication::Interpolation {
  pcg_context *_c;

 public:
  explicit GpuInterpolation(pcg_context *c) : _c(c) {}
  void interpolateSolution(const tarch::la::Vector<DIMENSIONS, int> &destinationSize,
                           const tarch::la::Vector<DIMENSIONS, int> &destinationOffset, peanoclaw::Patch &source,
                           peanoclaw::Patch &destination, bool interpolateToUOld, bool interpolateToCurrentTime,
                           bool useTimeUNewOrTimeUOld) override {
    pushTime(_c, source);
    pushTime(_c, destination);
    const int32_t size[2] = {destinationSize[0], destinationSize[1]};
    const int32_t off[2] = {destinationOffset[0], destinationOffset[1]};
    check(pcg_interpolate_solution(_c, size, off, deviceId(source), deviceId(destination), interpolateToUOld,
                                   interpolateToCurrentTime, useTimeUNewOrTimeUOld, 0),
          "pcg_interpolate_solution");
  }
};

class GpuRestriction : public peanoclaw::interSubgridCommunication::Restriction {
  pcg_context *_c;

 public:
  explicit GpuRestriction(pcg_context *c) : _c(c) {}
  void restrictSolution(peanoclaw::Patch &source, peanoclaw::Patch &destination,
                        bool restrictOnlyOverlappedRegions) override {
    pushTime(_c, source);
    pushTime(_c, destination);
    check(pcg_restrict_solution(_c, deviceId(source), deviceId(destination), restrictOnlyOverlappedRegions, 0),
          "pcg_restrict_solution");
  }
};

class GpuFluxCorrection : public peanoclaw::interSubgridCommunication::FluxCorrection {
  pcg_context *_c;

 public:
  explicit GpuFluxCorrection(pcg_context *c) : _c(c) {}
  void applyCorrection(Patch &finePatch, Patch &coarsePatch, int dimension, int direction) const override {
    pushTime(_c, finePatch);
    pushTime(_c, coarsePatch);
    check(pcg_apply_flux_correction(_c, deviceId(finePatch), deviceId(coarsePatch), dimension, direction),
          "pcg_apply_flux_correction");
  }
  // Numerics::computeFlux uses g = 1 (Numerics.h:198)
  void computeFluxes(Patch &subgrid) const override {
    check(pcg_compute_fluxes(_c, deviceId(subgrid), 1.0), "pcg_compute_fluxes");
  }
};

}  // namespace

pcg_context *gpuContext() { return g_context; }

GpuSWEKernel::GpuSWEKernel(pcg_context *context, const GpuRefinementCriterion &criterion)
    : Numerics(new peanoclaw::interSubgridCommunication::DefaultTransfer(), new GpuInterpolation(context),
               new GpuRestriction(context), new GpuFluxCorrection(context)),
      _context(context),
      _criterion(criterion) {
  if (!context) throw std::runtime_error("GpuSWEKernel: null library context");
  g_context = context;
}

GpuSWEKernel::~GpuSWEKernel() {
  if (g_context == _context) g_context = nullptr;
}

// SWEKernel::addPatchToSolution is empty (SWEKernel.cpp:173-174): output is
// gathered from the device (pcg_gather_cells) instead.
void GpuSWEKernel::addPatchToSolution(Patch &) {}

// SWEKernel::initializePatch lets the scenario write the initial state
// (SWEKernel.cpp:111-119); here the scenario writes it into the
// CellDescription's host vector (reference layout) and it is uploaded.
void GpuSWEKernel::initializePatch(Patch &patch) {
  peanoclaw::records::CellDescription &cd = patch.getCellDescription();
  if (!cd.hostData) throw std::runtime_error("initializePatch: the subgrid has no host data to upload");
  check(pcg_patch_upload(_context, deviceId(patch), cd.hostData->data(), (int64_t)cd.hostData->size()),
        "pcg_patch_upload");
  pushTime(_context, patch);
}

void GpuSWEKernel::transferGhostlayer(const tarch::la::Vector<DIMENSIONS, int> &size,
                                      const tarch::la::Vector<DIMENSIONS, int> &sourceOffset,
                                      const tarch::la::Vector<DIMENSIONS, int> &destinationOffset,
                                      peanoclaw::Patch &source, peanoclaw::Patch &destination) const {
  pushTime(_context, source);
  pushTime(_context, destination);
  const int32_t s[2] = {size[0], size[1]}, so[2] = {sourceOffset[0], sourceOffset[1]};
  const int32_t dof[2] = {destinationOffset[0], destinationOffset[1]};
  check(pcg_transfer_ghostlayer(_context, s, so, dof, deviceId(source), deviceId(destination)),
        "pcg_transfer_ghostlayer");
}

// SWEKernel::interpolateSolution: interpolation of the surface h + b
// (SWEKernel.cpp:239-286).
void GpuSWEKernel::interpolateSolution(const tarch::la::Vector<DIMENSIONS, int> &destinationSize,
                                       const tarch::la::Vector<DIMENSIONS, int> &destinationOffset,
                                       peanoclaw::Patch &source, peanoclaw::Patch &destination,
                                       bool interpolateToUOld, bool interpolateToCurrentTime,
                                       bool useTimeUNewOrTimeUOld) const {
  pushTime(_context, source);
  pushTime(_context, destination);
  const int32_t size[2] = {destinationSize[0], destinationSize[1]};
  const int32_t off[2] = {destinationOffset[0], destinationOffset[1]};
  check(pcg_interpolate_solution(_context, size, off, deviceId(source), deviceId(destination), interpolateToUOld,
                                 interpolateToCurrentTime, useTimeUNewOrTimeUOld, 1),
        "pcg_interpolate_solution");
}

// SWEKernel::restrictSolution: restriction of the surface h + b
// (SWEKernel.cpp:288-307).
void GpuSWEKernel::restrictSolution(peanoclaw::Patch &source, peanoclaw::Patch &destination,
                                    bool restrictOnlyOverlappedRegions) const {
  pushTime(_context, source);
  pushTime(_context, destination);
  check(pcg_restrict_solution(_context, deviceId(source), deviceId(destination), restrictOnlyOverlappedRegions, 1),
        "pcg_restrict_solution");
}

// SWEKernel::postProcessRestriction (SWEKernel.cpp:309-316).
void GpuSWEKernel::postProcessRestriction(peanoclaw::Patch &destination, bool) const {
  check(pcg_post_process_restriction(_context, deviceId(destination)), "pcg_post_process_restriction");
}

void GpuSWEKernel::fillBoundaryLayer(Patch &subgrid, int dimension, bool setUpper) {
  check(pcg_fill_boundary_layer(_context, deviceId(subgrid), dimension, setUpper ? 1 : 0), "pcg_fill_boundary_layer");
}

// SWEKernel::solveTimestep (SWEKernel.cpp:125-167): the device solves uOld
// (+ ghost layer) with dt = min(CFL dt, maximumTimestepSize), swaps, and
// advances its time record, which becomes the subgrid's time interval.  The
// block is not split dimension by dimension and the boundary flags do not
// change the solve, as in the reference's accumulation block.
void GpuSWEKernel::solveTimestep(Patch &subgrid, double maximumTimestepSize, bool,
                                 tarch::la::Vector<DIMENSIONS_TIMES_TWO, bool>) {
  pushTime(_context, subgrid);
  check(pcg_solve_timestep(_context, deviceId(subgrid), maximumTimestepSize, nullptr, nullptr),
        "pcg_solve_timestep");
  pullTime(_context, subgrid);
}

tarch::la::Vector<DIMENSIONS, double> GpuSWEKernel::getDemandedMeshWidth(Patch &patch, bool) {
  const int32_t id = deviceId(patch);
  double value = 0.0;
  check(pcg_refinement_criterion(_context, 1, &id, _criterion.kind, &value), "pcg_refinement_criterion");
  if (value > _criterion.threshold) return tarch::la::Vector<DIMENSIONS, double>(_criterion.minimalMeshWidth);
  if (value < _criterion.threshold) return tarch::la::Vector<DIMENSIONS, double>(_criterion.maximalMeshWidth);
  return patch.getSubcellSize();
}

void GpuSWEKernel::update(Patch &finePatch) {
  if (_update) _update(finePatch);
}

void GpuSWEKernel::allocatePatch(peanoclaw::records::CellDescription &cd) {
  pcg_patch_desc d;
  d.nx = cd.subdivisionFactor[0];
  d.ny = cd.subdivisionFactor[1];
  d.ghost = cd.ghostlayerWidth;
  d.nq = cd.unknownsPerSubcell;
  d.np_wo = cd.numberOfParametersWithoutGhostlayerPerSubcell;
  d.np_w = cd.numberOfParametersWithGhostlayerPerSubcell;
  d.level = cd.level;
  d.flags = flagsOf(cd);
  for (int k = 0; k < 2; k++) {
    d.pos[k] = cd.position[k];
    d.size[k] = cd.size[k];
  }
  int32_t id = -1;
  check(pcg_patch_alloc(_context, &d, &id), "pcg_patch_alloc");
  cd.uIndex = id;
  Patch patch(cd);
  pushTime(_context, patch);
}

void GpuSWEKernel::freePatch(peanoclaw::records::CellDescription &cd) {
  if (cd.uIndex < 0) return;
  check(pcg_patch_free(_context, cd.uIndex), "pcg_patch_free");
  cd.uIndex = -1;
}

void GpuSWEKernel::updatePatchState(Patch &patch) {
  check(pcg_patch_set_desc_flags(_context, deviceId(patch), flagsOf(patch.getCellDescription())),
        "pcg_patch_set_desc_flags");
}

}  // namespace native

// DefaultTransfer for device subgrids (DefaultTransfer.cpph:15-127): the
// operations SolveTimestep::enterCell and the compositor issue directly.
namespace interSubgridCommunication {

void DefaultTransfer::transferGhostlayer(const tarch::la::Vector<DIMENSIONS, int> &size,
                                         const tarch::la::Vector<DIMENSIONS, int> &sourceOffset,
                                         const tarch::la::Vector<DIMENSIONS, int> &destinationOffset,
                                         peanoclaw::Patch &source, peanoclaw::Patch &destination) {
  pcg_context *c = native::gpuContext();
  if (!c) throw std::runtime_error("DefaultTransfer: no GPU numerics object");
  native::pushTime(c, source);
  native::pushTime(c, destination);
  const int32_t s[2] = {size[0], size[1]}, so[2] = {sourceOffset[0], sourceOffset[1]};
  const int32_t dof[2] = {destinationOffset[0], destinationOffset[1]};
  native::check(pcg_transfer_ghostlayer(c, s, so, dof, native::deviceId(source), native::deviceId(destination)),
                "pcg_transfer_ghostlayer");
}

void DefaultTransfer::copyUNewToUOld(peanoclaw::Patch &subgrid) {
  pcg_context *c = native::gpuContext();
  if (!c) throw std::runtime_error("DefaultTransfer: no GPU numerics object");
  native::check(pcg_copy_unew_to_uold(c, native::deviceId(subgrid)), "pcg_copy_unew_to_uold");
}

void DefaultTransfer::swapUNewAndUOld(peanoclaw::Patch &subgrid) {
  pcg_context *c = native::gpuContext();
  if (!c) throw std::runtime_error("DefaultTransfer: no GPU numerics object");
  native::check(pcg_swap_unew_and_uold(c, native::deviceId(subgrid)), "pcg_swap_unew_and_uold");
}

}  // namespace interSubgridCommunication
}  // namespace peanoclaw
