/* Stand-in for the reference's geometry header when building the reference
 * core without libctl (an external, unvendored dependency).  The core uses
 * only the chunk-cost model from it (structure.cpp, vec.cpp get_cost); with
 * fragment_stats::resolution == 0 that model is never consulted, so the
 * stand-in returns a zero cost.  Test infrastructure only. */
#ifndef MEEP_GEOM_H
#define MEEP_GEOM_H
#include "meep.hpp"

struct geom_box {
  double low[3], high[3];
};

namespace meep_geom {
struct fragment_stats {
  static double resolution;
  static bool split_chunks_evenly;
  explicit fragment_stats(geom_box &) {}
  void compute() {}
  double cost() const { return 0.0; }
};
geom_box gv2box(const meep::volume &v);
} // namespace meep_geom
#endif
