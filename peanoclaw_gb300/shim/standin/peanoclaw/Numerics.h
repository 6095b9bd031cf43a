// Stand-in for peanoclaw/Numerics.h (src/peanoclaw/Numerics.h:30-204 in the
// reference): the numerics plugin interface with the reference's virtual
// signatures.  Peano 3 and the PeanoClaw build are not available to this
// repository, so the GPU plugin (GpuSWEKernel) is compiled here against this
// and the other stand-ins under standin/ (Patch, TimeIntervals, the three
// strategy interfaces, DefaultTransfer, tarch::la::Vector, Dimensions);
// inside PeanoClaw it compiles against the real headers instead.  The
// non-pure virtuals delegate to the strategy objects, which the Numerics
// object owns and deletes (Numerics.cpp:11-100).
#ifndef PEANOCLAW_NUMERICS_H_
#define PEANOCLAW_NUMERICS_H_

#include "peanoclaw/interSubgridCommunication/DefaultTransfer.h"
#include "peanoclaw/interSubgridCommunication/FluxCorrection.h"
#include "peanoclaw/interSubgridCommunication/Interpolation.h"
#include "peanoclaw/interSubgridCommunication/Restriction.h"
#include "tarch/la/Vector.h"

namespace peanoclaw {
class Patch;

class Numerics {
 private:
  peanoclaw::interSubgridCommunication::DefaultTransfer *_transfer;
  peanoclaw::interSubgridCommunication::Interpolation *_interpolation;
  peanoclaw::interSubgridCommunication::Restriction *_restriction;
  peanoclaw::interSubgridCommunication::FluxCorrection *_fluxCorrection;

 public:
  Numerics(peanoclaw::interSubgridCommunication::DefaultTransfer *transfer,
           peanoclaw::interSubgridCommunication::Interpolation *interpolation,
           peanoclaw::interSubgridCommunication::Restriction *restriction,
           peanoclaw::interSubgridCommunication::FluxCorrection *fluxCorrection)
      : _transfer(transfer), _interpolation(interpolation), _restriction(restriction),
        _fluxCorrection(fluxCorrection) {}

  virtual ~Numerics() {
    delete _transfer;
    delete _interpolation;
    delete _restriction;
    delete _fluxCorrection;
  }

  virtual void addPatchToSolution(Patch &patch) = 0;

  virtual void initializePatch(Patch &patch) = 0;

  virtual void transferGhostlayer(const tarch::la::Vector<DIMENSIONS, int> &size,
                                  const tarch::la::Vector<DIMENSIONS, int> &sourceOffset,
                                  const tarch::la::Vector<DIMENSIONS, int> &destinationOffset,
                                  peanoclaw::Patch &source, peanoclaw::Patch &destination) const {
    _transfer->transferGhostlayer(size, sourceOffset, destinationOffset, source, destination);
  }

  virtual void interpolateSolution(const tarch::la::Vector<DIMENSIONS, int> &destinationSize,
                                   const tarch::la::Vector<DIMENSIONS, int> &destinationOffset,
                                   peanoclaw::Patch &source, peanoclaw::Patch &destination, bool interpolateToUOld,
                                   bool interpolateToCurrentTime, bool useTimeUNewOrTimeUOld) const {
    _interpolation->interpolateSolution(destinationSize, destinationOffset, source, destination, interpolateToUOld,
                                        interpolateToCurrentTime, useTimeUNewOrTimeUOld);
  }

  virtual void restrictSolution(peanoclaw::Patch &source, peanoclaw::Patch &destination,
                                bool restrictOnlyOverlappedRegions) const {
    _restriction->restrictSolution(source, destination, restrictOnlyOverlappedRegions);
  }

  virtual void postProcessRestriction(peanoclaw::Patch &destination, bool restrictOnlyOverlappedRegions) const {}

  virtual void applyFluxCorrection(Patch &sourceSubgrid, Patch &destinationSubgrid, int dimension,
                                   int direction) const {
    _fluxCorrection->applyCorrection(sourceSubgrid, destinationSubgrid, dimension, direction);
  }

  virtual void computeFluxes(Patch &subgrid) const { _fluxCorrection->computeFluxes(subgrid); }

  virtual void fillBoundaryLayer(Patch &subgrid, int dimension, bool setUpper) = 0;

  virtual void solveTimestep(Patch &subgrid, double maximumTimestepSize, bool useDimensionalSplitting,
                             tarch::la::Vector<DIMENSIONS_TIMES_TWO, bool> domainBoundaryFlags) = 0;

  virtual tarch::la::Vector<DIMENSIONS, double> getDemandedMeshWidth(Patch &patch, bool isInitializing) = 0;

  virtual void update(Patch &finePatch) {}

  virtual int getNumberOfUnknownsPerCell() const = 0;

  virtual int getNumberOfParameterFieldsWithoutGhostlayer() const = 0;

  virtual int getNumberOfParameterFieldsWithGhostlayer() const = 0;

  virtual int getGhostlayerWidth() const = 0;
};

}  // namespace peanoclaw
#endif
