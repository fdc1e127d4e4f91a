/* Material-grid permittivity: the design weights u on a rectilinear grid over
 * a block, interpolated to a point, projected, and mapped to eps (host and
 * device code; included by the CUDA engine and by the CPU oracle).
 *
 * Restated from the reference:
 *   mg_map / mg_interp   map_coordinates and linear_interpolate
 *                        (src/fields.cpp:759-806): cell-centred grid nodes,
 *                        mirror reflection at the faces
 *   mg_project           tanh_projection (src/meepgeom.cpp:497-502)
 *   mg_eps               epsilon_material_grid's diagonal eps
 *                        (src/meepgeom.cpp:569-581): eps1 + u (eps2 - eps1)
 *   mg_coords            the point's block coordinates in [0, 1], as
 *                        map_lattice_coordinates (src/meepgeom.cpp:447-451),
 *                        0 along a direction of zero extent
 *   mg_inside            an axis-aligned block's point test, |x - c| <= s/2
 *                        per direction (inclusive, as libctl's block test)
 * Only the diagonal of eps and the default grid type (one grid, no overlap
 * rule) without subpixel smoothing of the grid (do_averaging false, the
 * reference's default) are covered. */
#ifndef MEEP_GB300_MATGRID_HPP
#define MEEP_GB300_MATGRID_HPP

#include <cmath>

#ifdef __CUDACC__
#define MG_HD __host__ __device__ __forceinline__
#else
#define MG_HD inline
#endif

namespace mfd {

struct MatGridSpec {
  double center[3], size[3];
  int n[3];           // grid nodes per direction (1 along an unused direction)
  double beta, eta;   // projection
  double eps1[3], eps2[3];
};

MG_HD int mg_mirror(int i, int n) { return i >= n ? 2 * n - 1 - i : (i < 0 ? -1 - i : i); }

// node pair (i1, i2) and weight w of i2 along one direction (weight of i1 is 1 - w)
MG_HD void mg_map(double r, int n, int &i1, int &i2, double &w) {
  r = r < 0.0 ? -r : (r > 1.0 ? 1.0 - r : r);
  i1 = mg_mirror(int(r * n), n);
  double d = r * n - i1 - 0.5;
  i2 = mg_mirror(d >= 0.0 ? i1 + 1 : i1 - 1, n);
  w = fabs(d);
}

// linear interpolation of u (row-major [n0][n1][n2]) at block coordinates r
MG_HD double mg_interp(const double *u, const int n[3], const double r[3]) {
  int x1, x2, y1, y2, z1, z2;
  double dx, dy, dz;
  mg_map(r[0], n[0], x1, x2, dx);
  mg_map(r[1], n[1], y1, y2, dy);
  mg_map(r[2], n[2], z1, z2, dz);
#define MG_U(x, y, z) (u[((x) * n[1] + (y)) * n[2] + (z)])
  return (((MG_U(x1, y1, z1) * (1.0 - dx) + MG_U(x2, y1, z1) * dx) * (1.0 - dy) +
           (MG_U(x1, y2, z1) * (1.0 - dx) + MG_U(x2, y2, z1) * dx) * dy) *
              (1.0 - dz) +
          ((MG_U(x1, y1, z2) * (1.0 - dx) + MG_U(x2, y1, z2) * dx) * (1.0 - dy) +
           (MG_U(x1, y2, z2) * (1.0 - dx) + MG_U(x2, y2, z2) * dx) * dy) *
              dz);
#undef MG_U
}

MG_HD double mg_project(double u, double beta, double eta) {
  if (beta == 0) return u;
  if (u == eta) return 0.5;
  const double t = tanh(beta * eta);
  return (t + tanh(beta * (u - eta))) / (t + tanh(beta * (1 - eta)));
}

// d mg_project / du (0 for an infinite beta away from eta)
MG_HD double mg_project_deriv(double u, double beta, double eta) {
  if (beta == 0) return 1.0;
  if (!(beta < 1.7976931348623157e308)) return 0.0; // infinite (or NaN) beta
  const double th = tanh(beta * (u - eta));
  return beta * (1.0 - th * th) / (tanh(beta * eta) + tanh(beta * (1 - eta)));
}

MG_HD bool mg_inside(const MatGridSpec &g, const double x[3]) {
  for (int d = 0; d < 3; d++)
    if (!(fabs(x[d] - g.center[d]) <= 0.5 * g.size[d])) return false;
  return true;
}

MG_HD void mg_coords(const MatGridSpec &g, const double x[3], double r[3]) {
  for (int d = 0; d < 3; d++)
    r[d] = g.size[d] == 0 ? 0.0 : 0.5 + (x[d] - g.center[d]) / g.size[d];
}

MG_HD double mg_eps(const MatGridSpec &g, int d, double up) { return g.eps1[d] + up * (g.eps2[d] - g.eps1[d]); }

} // namespace mfd

#endif
