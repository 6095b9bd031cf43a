// Stand-in for peanoclaw/Patch.h: a transient view over one subgrid's
// CellDescription (geometry, refinement state, time interval, data index).
// In the GPU integration the data index uIndex names the device patch
// (pcg_patch_alloc) instead of a Peano DataHeap entry.
#ifndef PEANOCLAW_PATCH_H_
#define PEANOCLAW_PATCH_H_
#include <vector>

#include "peano/utils/Dimensions.h"
#include "peanoclaw/grid/TimeIntervals.h"
#include "tarch/la/Vector.h"

namespace peanoclaw {
namespace records {

// The fields of CellDescription (dastgen/CellDescription.def) that the
// numerics plugin reads.
struct CellDescription {
  tarch::la::Vector<DIMENSIONS, int> subdivisionFactor;
  int ghostlayerWidth = 1;
  int unknownsPerSubcell = 3;
  int numberOfParametersWithoutGhostlayerPerSubcell = 0;
  int numberOfParametersWithGhostlayerPerSubcell = 1;
  tarch::la::Vector<DIMENSIONS, double> position;
  tarch::la::Vector<DIMENSIONS, double> size;
  int level = 0;
  bool isLeaf = true;
  bool isVirtual = false;
  double time = 0.0, timestepSize = 0.0, estimatedNextTimestepSize = 0.0;
  double minimalNeighborTime = 0.0, maximalNeighborTimestep = 0.0;
  tarch::la::Vector<DIMENSIONS, double> lowerNeighboringGhostlayerBounds;
  tarch::la::Vector<DIMENSIONS, double> upperNeighboringGhostlayerBounds;
  int uIndex = -1;
  // initial data of the subgrid in the reference layout, written by a
  // scenario on the host and uploaded by Numerics::initializePatch
  std::vector<double> *hostData = nullptr;
  tarch::la::Vector<DIMENSIONS, double> demandedMeshWidth;
};

}  // namespace records

class Patch {
  records::CellDescription *_cellDescription;

 public:
  explicit Patch(records::CellDescription &cellDescription) : _cellDescription(&cellDescription) {}
  const tarch::la::Vector<DIMENSIONS, double> getSize() const { return _cellDescription->size; }
  const tarch::la::Vector<DIMENSIONS, double> getPosition() const { return _cellDescription->position; }
  int getUnknownsPerSubcell() const { return _cellDescription->unknownsPerSubcell; }
  int getNumberOfParametersWithoutGhostlayerPerSubcell() const {
    return _cellDescription->numberOfParametersWithoutGhostlayerPerSubcell;
  }
  int getNumberOfParametersWithGhostlayerPerSubcell() const {
    return _cellDescription->numberOfParametersWithGhostlayerPerSubcell;
  }
  tarch::la::Vector<DIMENSIONS, int> getSubdivisionFactor() const { return _cellDescription->subdivisionFactor; }
  int getGhostlayerWidth() const { return _cellDescription->ghostlayerWidth; }
  int getLevel() const { return _cellDescription->level; }
  tarch::la::Vector<DIMENSIONS, double> getSubcellSize() const {
    tarch::la::Vector<DIMENSIONS, double> h;
    for (int d = 0; d < DIMENSIONS; d++) h[d] = _cellDescription->size[d] / _cellDescription->subdivisionFactor[d];
    return h;
  }
  int getUIndex() const { return _cellDescription->uIndex; }
  bool isLeaf() const { return _cellDescription->isLeaf; }
  bool isVirtual() const { return _cellDescription->isVirtual; }
  grid::TimeIntervals getTimeIntervals() const { return grid::TimeIntervals(_cellDescription); }
  tarch::la::Vector<DIMENSIONS, double> getLowerNeighboringGhostlayerBounds() const {
    return _cellDescription->lowerNeighboringGhostlayerBounds;
  }
  tarch::la::Vector<DIMENSIONS, double> getUpperNeighboringGhostlayerBounds() const {
    return _cellDescription->upperNeighboringGhostlayerBounds;
  }
  void setDemandedMeshWidth(const tarch::la::Vector<DIMENSIONS, double> &w) { _cellDescription->demandedMeshWidth = w; }
  tarch::la::Vector<DIMENSIONS, double> getDemandedMeshWidth() const { return _cellDescription->demandedMeshWidth; }
  records::CellDescription &getCellDescription() { return *_cellDescription; }
};

namespace grid {
inline double TimeIntervals::getCurrentTime() const { return _cellDescription->time; }
inline void TimeIntervals::setCurrentTime(double t) { _cellDescription->time = t; }
inline double TimeIntervals::getTimestepSize() const { return _cellDescription->timestepSize; }
inline void TimeIntervals::setTimestepSize(double dt) { _cellDescription->timestepSize = dt; }
inline double TimeIntervals::getEstimatedNextTimestepSize() const {
  return _cellDescription->estimatedNextTimestepSize;
}
inline void TimeIntervals::setEstimatedNextTimestepSize(double dt) { _cellDescription->estimatedNextTimestepSize = dt; }
inline double TimeIntervals::getTimeUOld() const { return _cellDescription->time; }
inline double TimeIntervals::getTimeUNew() const { return _cellDescription->time + _cellDescription->timestepSize; }
inline void TimeIntervals::advanceInTime() { _cellDescription->time += _cellDescription->timestepSize; }
inline double TimeIntervals::getMinimalFineGridTime() const { return _cellDescription->minimalNeighborTime; }
inline double TimeIntervals::getMaximalFineGridTimestep() const { return _cellDescription->maximalNeighborTimestep; }
}  // namespace grid

}  // namespace peanoclaw
#endif
