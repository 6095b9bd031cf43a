// Stand-in for peanoclaw/interSubgridCommunication/FluxCorrection.h: the
// flux-correction strategy interface (FluxCorrection.h:38-45).
#ifndef PEANOCLAW_INTERSUBGRIDCOMMUNICATION_FLUXCORRECTION_H_
#define PEANOCLAW_INTERSUBGRIDCOMMUNICATION_FLUXCORRECTION_H_

namespace peanoclaw {
class Patch;
namespace interSubgridCommunication {

class FluxCorrection {
 public:
  virtual ~FluxCorrection() {}
  virtual void applyCorrection(Patch &finePatch, Patch &coarsePatch, int dimension, int direction) const = 0;
  virtual void computeFluxes(Patch &subgrid) const = 0;
};

}  // namespace interSubgridCommunication
}  // namespace peanoclaw
#endif
