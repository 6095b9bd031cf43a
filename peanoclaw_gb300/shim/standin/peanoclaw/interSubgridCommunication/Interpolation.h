// Stand-in for peanoclaw/interSubgridCommunication/Interpolation.h:
// the interpolation strategy interface (Interpolation.h:64-72).
#ifndef PEANOCLAW_INTERSUBGRIDCOMMUNICATION_INTERPOLATION_H_
#define PEANOCLAW_INTERSUBGRIDCOMMUNICATION_INTERPOLATION_H_
#include "peano/utils/Dimensions.h"
#include "tarch/la/Vector.h"

namespace peanoclaw {
class Patch;
namespace interSubgridCommunication {

class Interpolation {
 public:
  virtual ~Interpolation() {}
  virtual void interpolateSolution(const tarch::la::Vector<DIMENSIONS, int> &destinationSize,
                                   const tarch::la::Vector<DIMENSIONS, int> &destinationOffset,
                                   peanoclaw::Patch &source, peanoclaw::Patch &destination, bool interpolateToUOld,
                                   bool interpolateToCurrentTime, bool useTimeUNewOrTimeUOld) = 0;
};

}  // namespace interSubgridCommunication
}  // namespace peanoclaw
#endif
