// Stand-in for peanoclaw/interSubgridCommunication/Restriction.h: the
// restriction strategy interface (Restriction.h:35-39).
#ifndef PEANOCLAW_INTERSUBGRIDCOMMUNICATION_RESTRICTION_H_
#define PEANOCLAW_INTERSUBGRIDCOMMUNICATION_RESTRICTION_H_

namespace peanoclaw {
class Patch;
namespace interSubgridCommunication {

class Restriction {
 public:
  virtual ~Restriction() {}
  virtual void restrictSolution(peanoclaw::Patch &source, peanoclaw::Patch &destination,
                                bool restrictOnlyOverlappedRegions) = 0;
};

}  // namespace interSubgridCommunication
}  // namespace peanoclaw
#endif
