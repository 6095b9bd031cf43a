// Stand-in for peanoclaw/grid/TimeIntervals.h: the time interval of a
// subgrid (current time, timestep size, CFL estimate; the neighbour interval
// of a virtual subgrid), a view over its CellDescription.
#ifndef PEANOCLAW_GRID_TIMEINTERVALS_H_
#define PEANOCLAW_GRID_TIMEINTERVALS_H_

namespace peanoclaw {
namespace records {
struct CellDescription;
}
namespace grid {

class TimeIntervals {
  records::CellDescription *_cellDescription;

 public:
  explicit TimeIntervals(records::CellDescription *cellDescription) : _cellDescription(cellDescription) {}
  double getCurrentTime() const;
  void setCurrentTime(double currentTime);
  double getTimestepSize() const;
  void setTimestepSize(double timestepSize);
  double getEstimatedNextTimestepSize() const;
  void setEstimatedNextTimestepSize(double estimatedNextTimestepSize);
  // uOld / uNew times of a leaf (TimeIntervals.cpp:102-123)
  double getTimeUOld() const;
  double getTimeUNew() const;
  // time += timestep size
  void advanceInTime();
  // the interval a virtual subgrid holds (minimal time and maximal
  // timestep of its neighbours / fine grids)
  double getMinimalFineGridTime() const;
  double getMaximalFineGridTimestep() const;
};

}  // namespace grid
}  // namespace peanoclaw
#endif
