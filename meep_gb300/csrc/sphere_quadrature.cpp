// Quadrature points on the unit sphere (1-D, 2-D, 3-D) for the normal-vector
// estimate of subpixel averaging; the table the reference generates with its
// sphere_quad program (src/sphere-quad.cpp) and includes as sphere-quad.h.
//
// 3-D: A. D. McLaren, "Optimal Numerical Integration on a Sphere", Math.
// Comp. 17 (1963) 361-383, the 50-point formula of degree 11 (Stroud,
// "Approximate Calculation of Multiple Integrals", formula U3:11-1): four
// orbits of the octahedral group with weights 9216, 16384, 15309 and 14641
// over 725760.  The orbit members are enumerated as the reference does (sign
// flips x outermost, then the cyclic shifts (x,y,z) -> (z,x,y)), because the
// ordering step below breaks ties by position.
// 2-D: 12 equally spaced points on the circle, weight 1/12.  1-D: the poles.
// Each 2-D/3-D list is then reordered greedily: position i takes the point
// whose smallest squared distance (rounded to float) to points 0..i-1 is
// largest, ties going to the larger sum of those distances, then to the
// earlier point.
#include <cmath>
#include <utility>

#include "subpixel.hpp"

namespace mgb_subpixel {
namespace {

struct Builder {
  double (*pt)[4];
  int n = 0;
  void add(double x, double y, double z, double w) {
    pt[n][0] = x;
    pt[n][1] = y;
    pt[n][2] = z;
    pt[n][3] = w;
    n++;
  }
  // the three cyclic shifts of (x, y, z), starting with (z, x, y)
  void add_cyclic(double x, double y, double z, double w) {
    for (int r = 0; r < 3; r++) {
      const double t = z;
      z = y;
      y = x;
      x = t;
      add(x, y, z, w);
    }
  }
};

void greedy_order(double (*p)[4], int n) {
  for (int i = 1; i < n; ++i) {
    double best_min = 0, best_sum = 0;
    int jbest = i;
    for (int j = i; j < n; ++j) {
      double dmin = 1e20, dsum = 0;
      for (int k = 0; k < i; ++k) {
        const double dx = p[k][0] - p[j][0], dy = p[k][1] - p[j][1], dz = p[k][2] - p[j][2];
        const double d2 = float(dx * dx + dy * dy + dz * dz);
        dmin = d2 < dmin ? d2 : dmin;
        dsum += d2;
      }
      if (dmin > best_min || (dmin == best_min && dsum > best_sum)) {
        best_min = dmin;
        best_sum = dsum;
        jbest = j;
      }
    }
    for (int c = 0; c < 4; c++)
      std::swap(p[i][c], p[jbest][c]);
  }
}

SphereQuad build() {
  SphereQuad q{};
  q.n[0] = 2;
  q.n[1] = 12;
  q.n[2] = 50;
  // 1-D
  Builder b1{q.pt[0]};
  b1.add(0, 0, 1, 0.5);
  b1.add(0, 0, -1, 0.5);
  // 2-D
  Builder b2{q.pt[1]};
  const double pi = 3.141592653589793238462643383279502884197;
  for (int i = 0; i < 12; ++i)
    b2.add(std::cos(2 * i * pi / 12), std::sin(2 * i * pi / 12), 0.0, 1.0 / 12);
  greedy_order(q.pt[1], 12);
  // 3-D
  Builder b3{q.pt[2]};
  const double den = 725760.0;
  const double sgn[2] = {-1.0, 1.0};
  for (int i = 0; i < 2; ++i) // (+-1, 0, 0)
    b3.add_cyclic(sgn[i], 0, 0, 9216 / den);
  const double h = std::sqrt(0.5);
  for (int i = 0; i < 2; ++i) // (+-h, +-h, 0)
    for (int j = 0; j < 2; ++j)
      b3.add_cyclic(sgn[i] * h, sgn[j] * h, 0, 16384 / den);
  const double t = std::sqrt(1.0 / 3.0);
  for (int i = 0; i < 2; ++i) // (+-t, +-t, +-t)
    for (int j = 0; j < 2; ++j)
      for (int k = 0; k < 2; ++k)
        b3.add(sgn[i] * t, sgn[j] * t, sgn[k] * t, 15309 / den);
  const double u = std::sqrt(1.0 / 11.0), u3 = 3 * u;
  for (int i = 0; i < 2; ++i) // (+-u, +-u, +-3u)
    for (int j = 0; j < 2; ++j)
      for (int k = 0; k < 2; ++k)
        b3.add_cyclic(sgn[i] * u, sgn[j] * u, sgn[k] * u3, 14641 / den);
  greedy_order(q.pt[2], 50);
  return q;
}

} // namespace

const SphereQuad &sphere_quadrature() {
  static const SphereQuad q = build();
  return q;
}

} // namespace mgb_subpixel
