/* Definitions for the stand-in geometry header (see meepgeom.hpp here). */
#include "meepgeom.hpp"

namespace meep_geom {
double fragment_stats::resolution = 0.0;
bool fragment_stats::split_chunks_evenly = true;
geom_box gv2box(const meep::volume &v) {
  geom_box b = {{0, 0, 0}, {0, 0, 0}};
  (void)v;
  return b;
}
} // namespace meep_geom
