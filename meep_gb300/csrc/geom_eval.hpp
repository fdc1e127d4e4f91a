// Point-in-object tests of the geometry the Python front end passes down
// (blocks, spheres, cylinders), shared by the host (meep_pyshim.cpp) and the
// device subpixel-averaging kernel (mfd_subpixel.cu) so that both see the
// same material at every point.  The reference's Python layer evaluates these
// shapes through libctl (python/geom.py -> src/meepgeom.cpp); the tests here
// are the plain definitions: a block is axis-aligned with edges `size`, a
// sphere has `radius`, a cylinder has `radius`, `height` and unit `axis`.
// Coordinates of directions absent from the grid are 0.
#ifndef MGB_GEOM_EVAL_HPP_
#define MGB_GEOM_EVAL_HPP_

#include <cmath>

#if defined(__CUDACC__)
#define MGB_GHD __host__ __device__
#else
#define MGB_GHD
#endif

namespace mgb_geom {

template <class O> MGB_GHD inline bool contains(const O &o, const double r[3]) {
  double p[3];
  for (int d = 0; d < 3; d++)
    p[d] = r[d] - o.center[d];
  if (o.kind == 0) {
    for (int d = 0; d < 3; d++)
      if (std::fabs(p[d]) > 0.5 * o.size[d]) return false;
    return true;
  }
  if (o.kind == 1) return p[0] * p[0] + p[1] * p[1] + p[2] * p[2] <= o.radius * o.radius;
  const double h = p[0] * o.axis[0] + p[1] * o.axis[1] + p[2] * o.axis[2];
  if (std::fabs(h) > 0.5 * o.height) return false;
  double q2 = 0;
  for (int d = 0; d < 3; d++) {
    const double q = p[d] - h * o.axis[d];
    q2 += q * q;
  }
  return q2 <= o.radius * o.radius;
}

// index of the last object containing r, -1 if none (later objects take
// precedence, as in libctl)
template <class O> MGB_GHD inline int object_at(const O *objs, int nobj, const double r[3]) {
  for (int q = nobj - 1; q >= 0; q--)
    if (contains(objs[q], r)) return q;
  return -1;
}

} // namespace mgb_geom

#endif
