// Subpixel averaging of the permittivity: the effective inverse-permittivity
// row of one pixel from a scalar material function, host and device.
//
// Follows the reference's default (non-libctl) averaging:
//   material_function::normal_vector     src/anisotropic_averaging.cpp:60-85
//     gradient of chi1p1 by a quadrature over the sphere of one pixel
//     diameter; uniform when the first 2^dims quadrature points agree
//   material_function::eff_chi1inv_row   src/anisotropic_averaging.cpp:87-208
//     mean eps and mean 1/eps over the pixel by a ms^dims point grid, ms = 10
//     doubled until either mean moves by less than tol (relative) or the
//     evaluation count passes maxeval; then the row of
//     P (<1/eps> - 1/<eps>) + I / <eps>,  P = n n^T, n the unit normal
//   the quadrature table                 src/sphere-quad.cpp
//     1-D: the two poles; 2-D: 12 points on the circle; 3-D: McLaren's
//     50-point 11th-degree formula (Stroud U3:11-1); each list ordered
//     greedily so every point is as far as possible from the previous ones.
//
// The arithmetic is written out in the reference's operation order so that
// the row is bit-identical to the reference's (IEEE double, no contraction:
// host code with -ffp-contract=off, device code with --fmad=false).
#ifndef MGB_SUBPIXEL_HPP_
#define MGB_SUBPIXEL_HPP_

#include <cmath>

#if defined(__CUDACC__)
#define MGB_HD __host__ __device__
#else
#define MGB_HD
#endif

namespace mgb_subpixel {

constexpr int MAXQ = 50;

// quadrature points (x, y, z, weight) per dimension 1, 2, 3
struct SphereQuad {
  int n[3];
  double pt[3][MAXQ][4];
};

// the table, generated once (sphere_quadrature.cpp)
const SphereQuad &sphere_quadrature();

/* Pixels are boxes [lo, hi] of a dim-dimensional grid (dim 1: only z is
   used; dim 2: x and y; dim 3: x, y, z); chi(p) returns chi1p1 at the point
   p[3] (unused coordinates 0). */

// Gradient of chi1p1 by the sphere quadrature (zero where the first 2^dim
// quadrature points see the same value).
template <class Chi>
MGB_HD void normal_vector(int dim, const double lo[3], const double hi[3], const SphereQuad &sq, Chi chi,
                          double grad[3]) {
  const bool act[3] = {dim >= 2, dim >= 2, dim != 2};
  double cen[3] = {0, 0, 0};
  double R = 0.0;
  for (int d = 0; d < 3; d++) {
    grad[d] = 0.0;
    if (!act[d]) continue;
    cen[d] = (hi[d] + lo[d]) * 0.5;
    const double e = hi[d] - lo[d];
    R = R < e ? e : R;
  }
  const int nq = sq.n[dim - 1];
  const int min_iters = 1 << dim;
  double prev = 0;
  bool uniform = true;
  for (int i = 0; i < nq; ++i) {
    const double *q = sq.pt[dim - 1][i];
    double p[3] = {0, 0, 0};
    for (int d = 0; d < 3; d++)
      if (act[d]) p[d] = q[d] * R + cen[d];
    const double v = chi(p);
    if (i > 0 && i < min_iters) {
      if (v != prev) uniform = false;
      if (i == min_iters - 1 && uniform) {
        grad[0] = grad[1] = grad[2] = 0.0;
        return;
      }
    }
    prev = v;
    const double wv = q[3] * v;
    for (int d = 0; d < 3; d++)
      if (act[d]) grad[d] += (p[d] - cen[d]) * wv;
  }
}

// Row cdir (0, 1, 2) of the effective inverse permittivity of the pixel;
// maxeval == 0: no averaging.
template <class Chi>
MGB_HD void eff_chi1inv_row(int dim, int cdir, const double lo[3], const double hi[3], double tol, int maxeval,
                            const SphereQuad &sq, Chi chi, double row[3]) {
  const bool act[3] = {dim >= 2, dim >= 2, dim != 2};
  double cen[3] = {0, 0, 0}, ext[3] = {0, 0, 0};
  for (int d = 0; d < 3; d++)
    if (act[d]) {
      cen[d] = (hi[d] + lo[d]) * 0.5;
      ext[d] = hi[d] - lo[d];
    }
  double meps = 1, minveps = 1;
  double grad[3];
  double gabs = 0;
  if (!maxeval) goto trivial;
  {
    normal_vector(dim, lo, hi, sq, chi, grad);
    double g2 = 0.0;
    for (int d = 0; d < 3; d++)
      if (act[d]) g2 += grad[d] * grad[d];
    gabs = std::sqrt(g2);
    if (gabs < 1e-8) goto trivial;

    // mean eps and mean 1/eps on refined grids
    int ms = 10, iter = 0;
    double old_meps = 0, old_minveps = 0;
    while (std::fabs(meps - old_meps) > tol * std::fabs(old_meps) &&
           std::fabs(minveps - old_minveps) > tol * std::fabs(old_minveps)) {
      old_meps = meps;
      old_minveps = minveps;
      meps = minveps = 0;
      const int n2 = dim >= 2 ? ms : 1, n3 = dim >= 3 ? ms : 1;
      for (int k = 0; k < n3; k++)
        for (int j = 0; j < n2; j++)
          for (int i = 0; i < ms; i++) {
            double p[3] = {0, 0, 0};
            if (dim == 1) p[2] = lo[2] + i * ext[2] / ms;
            else {
              p[0] = lo[0] + i * ext[0] / ms;
              p[1] = lo[1] + j * ext[1] / ms;
              if (dim == 3) p[2] = lo[2] + k * ext[2] / ms;
            }
            const double ep = chi(p);
            if (ep < 0) {
              if (dim != 1) goto trivial;
              // 1-D: the pixel-centre value, still along the normal
              meps = chi(cen);
              minveps = 1 / meps;
              goto done;
            }
            meps += ep;
            minveps += 1 / ep;
          }
      const int cnt = ms * n2 * n3;
      meps /= cnt;
      minveps /= cnt;
      ms *= 2;
      // the reference counts ms^3 (3-D) or ms^2 (1-D, 2-D) of the doubled ms
      if (maxeval && (iter += (dim == 3 ? ms * ms * ms : ms * ms)) >= maxeval) goto done;
    }
  }
done : {
  double n[3] = {0, 0, 0};
  const double inv = 1.0 / gabs;
  for (int d = 0; d < 3; d++)
    if (act[d]) n[d] = grad[d] * inv;
  for (int i = 0; i < 3; ++i)
    row[i] = n[cdir] * n[i] * (minveps - 1 / meps);
  row[cdir] += 1 / meps;
  return;
}
trivial:
  row[0] = row[1] = row[2] = 0.0;
  row[cdir] = 1 / chi(cen);
}

} // namespace mgb_subpixel

#endif
