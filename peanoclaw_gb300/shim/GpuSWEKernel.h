// GpuSWEKernel.h -- the GB300 SWE kernel as a peanoclaw::Numerics plugin.
//
// A drop-in for peanoclaw::native::SWEKernel (src/peanoclaw/native/
// SWEKernel.h:32-167 in the reference): every virtual of the Numerics
// interface forwards to one entry point of libpcg.so (include/pcg.h), on the
// device patch that the subgrid's CellDescription names in its uIndex.  The
// patch's time interval stays in the CellDescription, as in the reference;
// the plugin writes it to the device before every operation that reads
// times (transfers, interpolation, restriction, flux correction, the solve)
// and reads the device's record back after a solve.  Errors of the library
// are raised as std::runtime_error with the library's error text.
#ifndef PEANOCLAW_GB300_GPUSWEKERNEL_H_
#define PEANOCLAW_GB300_GPUSWEKERNEL_H_

#include <functional>

#include "pcg.h"
#include "peanoclaw/Numerics.h"
#include "peanoclaw/Patch.h"

namespace peanoclaw {
namespace native {

// Refinement criterion of the scenario (SWEScenario::computeDemandedMeshWidth):
// the device criterion `kind` (PCG_CRIT_*) above `threshold` demands the
// minimal mesh width, below it the maximal one (BreakingDam.cpp:85-139).
struct GpuRefinementCriterion {
  int kind = PCG_CRIT_DEPTH_GRADIENT;
  double threshold = 0.1;
  double minimalMeshWidth = 0.0;
  double maximalMeshWidth = 1.0;
};

class GpuSWEKernel : public peanoclaw::Numerics {
 public:
  // Takes the library context the subgrids live in (not owned); the
  // DefaultTransfer operations of the traversal use it too.
  GpuSWEKernel(pcg_context *context, const GpuRefinementCriterion &criterion);
  ~GpuSWEKernel() override;

  // -- Numerics interface
  void addPatchToSolution(Patch &patch) override;
  void initializePatch(Patch &patch) override;
  void transferGhostlayer(const tarch::la::Vector<DIMENSIONS, int> &size,
                          const tarch::la::Vector<DIMENSIONS, int> &sourceOffset,
                          const tarch::la::Vector<DIMENSIONS, int> &destinationOffset, peanoclaw::Patch &source,
                          peanoclaw::Patch &destination) const override;
  void interpolateSolution(const tarch::la::Vector<DIMENSIONS, int> &destinationSize,
                           const tarch::la::Vector<DIMENSIONS, int> &destinationOffset, peanoclaw::Patch &source,
                           peanoclaw::Patch &destination, bool interpolateToUOld, bool interpolateToCurrentTime,
                           bool useTimeUNewOrTimeUOld) const override;
  void restrictSolution(peanoclaw::Patch &source, peanoclaw::Patch &destination,
                        bool restrictOnlyOverlappedRegions) const override;
  void postProcessRestriction(peanoclaw::Patch &destination, bool restrictOnlyOverlappedRegions) const override;
  void fillBoundaryLayer(Patch &subgrid, int dimension, bool setUpper) override;
  void solveTimestep(Patch &subgrid, double maximumTimestepSize, bool useDimensionalSplitting,
                     tarch::la::Vector<DIMENSIONS_TIMES_TWO, bool> domainBoundaryFlags) override;
  tarch::la::Vector<DIMENSIONS, double> getDemandedMeshWidth(Patch &patch, bool isInitializing) override;
  void update(Patch &finePatch) override;
  int getNumberOfUnknownsPerCell() const override { return 3; }
  int getNumberOfParameterFieldsWithoutGhostlayer() const override { return 0; }
  int getNumberOfParameterFieldsWithGhostlayer() const override { return 1; }
  int getGhostlayerWidth() const override { return 1; }

  // -- device patches
  // Allocates the device patch of a subgrid (its CellDescription's geometry,
  // refinement state and time interval) and stores its id in uIndex.
  void allocatePatch(peanoclaw::records::CellDescription &cellDescription);
  void freePatch(peanoclaw::records::CellDescription &cellDescription);
  // After a subgrid became leaf / virtual: the device flags follow.
  void updatePatchState(Patch &patch);
  // Bathymetry update of a fine subgrid (SWEScenario::update; the reference
  // scenarios that set the ghost-layer bathymetry); none by default.
  void setUpdateCallback(std::function<void(Patch &)> callback) { _update = callback; }

  pcg_context *context() const { return _context; }

 private:
  pcg_context *_context;
  GpuRefinementCriterion _criterion;
  std::function<void(Patch &)> _update;
};

// The library context of the GPU numerics object the traversal's
// DefaultTransfer operations use (set by GpuSWEKernel's constructor).
pcg_context *gpuContext();

}  // namespace native
}  // namespace peanoclaw
#endif
