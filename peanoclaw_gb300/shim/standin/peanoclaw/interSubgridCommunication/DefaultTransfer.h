// Stand-in for peanoclaw/interSubgridCommunication/DefaultTransfer.h: the
// ghost-layer copy with time interpolation and the uNew / uOld transfers
// that SolveTimestep::enterCell issues directly (SolveTimestep.cpp:632-633).
// The definitions for device patches are in the plugin's GpuSWEKernel.cpp.
#ifndef PEANOCLAW_INTERSUBGRIDCOMMUNICATION_DEFAULTTRANSFER_H_
#define PEANOCLAW_INTERSUBGRIDCOMMUNICATION_DEFAULTTRANSFER_H_
#include "peano/utils/Dimensions.h"
#include "tarch/la/Vector.h"

namespace peanoclaw {
class Patch;
namespace interSubgridCommunication {

class DefaultTransfer {
 public:
  void transferGhostlayer(const tarch::la::Vector<DIMENSIONS, int> &size,
                          const tarch::la::Vector<DIMENSIONS, int> &sourceOffset,
                          const tarch::la::Vector<DIMENSIONS, int> &destinationOffset, peanoclaw::Patch &source,
                          peanoclaw::Patch &destination);
  void copyUNewToUOld(peanoclaw::Patch &subgrid);
  void swapUNewAndUOld(peanoclaw::Patch &subgrid);
};

}  // namespace interSubgridCommunication
}  // namespace peanoclaw
#endif
