// Homogeneous-medium Green's functions of the near-to-far transform, host and
// device: the E and H fields (6 complex values, Ex Ey Ez Hx Hy Hz) at x of a
// point current of complex amplitude f0 at x0, polarised along one axis, at
// frequency freq in a medium of scalar eps and mu.
//
// Follows the reference's
//   green3d   src/near2far.cpp:131-181   electric / magnetic dipole fields,
//             written for a current J = -i omega p (the usual dipole-moment
//             formulas divided by -i omega):
//               E (electric source) = F / eps * [t1 p + t2 (p.r) r],
//               H (electric source) = F / eps * t3 (r x p) / Z,
//             F = f0 k n / (4 pi r) exp(i (k r + pi/2)), n = sqrt(eps mu),
//             k = 2 pi freq n, Z = sqrt(mu / eps),
//             t1 = 1 - 1/(ikr) + 1/(ikr)^2, t2 = -1 + 3/(ikr) - 3/(ikr)^2,
//             t3 = 1 - 1/(ikr); a magnetic source swaps the roles (E from
//             -F/mu t3 (r x p) Z, H from F/mu [t1 p + t2 (p.r) r]).
//   green2d   src/near2far.cpp:201-245   line currents, Hankel functions
//             H_n = J_n + i Y_n of k r (out-of-plane and in-plane sources).
// The operations are written in the reference's order (complex products as
// (ac - bd, ad + bc)), so that a host build without contraction gives the
// reference's values up to the last bits of libm's sincos and Bessel
// functions.
#ifndef MGB_GREENS_HPP_
#define MGB_GREENS_HPP_

#include <cmath>

#if defined(__CUDACC__)
#define MGB_GRN __host__ __device__ __forceinline__
#else
#define MGB_GRN inline
#endif

namespace mgb_green {

struct cplx {
  double re, im;
};

MGB_GRN cplx cmul(cplx a, cplx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
MGB_GRN cplx cscale(cplx a, double s) { return {a.re * s, a.im * s}; }
MGB_GRN cplx cadd(cplx a, cplx b) { return {a.re + b.re, a.im + b.im}; }
MGB_GRN cplx csub(cplx a, cplx b) { return {a.re - b.re, a.im - b.im}; }

constexpr double PI = 3.141592653589793238462643383279502884;

// c0: 0..2 electric current along x, y, z; 3..5 magnetic along x, y, z.
// x, x0: 3 coordinates (the z coordinate unused in 2-D).  EH: 6 values.
MGB_GRN void green3d(cplx EH[6], const double x[3], double freq, double eps, double mu, const double x0[3], int c0,
                     cplx f0) {
  double rv[3] = {x[0] - x0[0], x[1] - x0[1], x[2] - x0[2]};
  const double r = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
  // vec / r multiplies by 1 / r (src/meep/vec.hpp:680-684)
  rv[0] = rv[0] * (1.0 / r);
  rv[1] = rv[1] * (1.0 / r);
  rv[2] = rv[2] * (1.0 / r);
  const double n = sqrt(eps * mu);
  const double k = 2 * PI * freq * n;
  const double kr = k * r;
  // 1/(ikr) = -i/(kr); 1/(ikr)^2 = 1/(-(kr)^2)
  const double ikr2 = -(kr) * (kr);
  const double inv_kr = 1.0 / kr;
  const double amp = k * n / (4 * PI * r);
  double sn, cs;
  const double ph = kr + PI * 0.5;
  sn = sin(ph);
  cs = cos(ph);
  cplx expfac = cmul(f0, cplx{amp * cs, amp * sn});
  const double Z = sqrt(mu / eps);
  const int d = c0 % 3;
  const double p[3] = {d == 0 ? 1.0 : 0.0, d == 1 ? 1.0 : 0.0, d == 2 ? 1.0 : 0.0};
  const double pdotr = p[0] * rv[0] + p[1] * rv[1] + p[2] * rv[2];
  const double rxp[3] = {rv[1] * p[2] - rv[2] * p[1], rv[2] * p[0] - rv[0] * p[2], rv[0] * p[1] - rv[1] * p[0]};
  // t1 = (1 - 1/ikr) + 1/ikr2; t2 = ((-1 + 3/ikr) - 3/ikr2) (p.r); t3 = 1 - 1/ikr
  const cplx t1 = {1.0 + 1.0 / ikr2, inv_kr};
  const cplx t2 = cscale(cplx{-1.0 - 3.0 / ikr2, -(3.0 / kr)}, pdotr);
  const cplx t3 = {1.0, inv_kr};
  const bool electric = c0 < 3;
  const double m = electric ? eps : mu;
  expfac = cplx{expfac.re / m, expfac.im / m};
  cplx A[3], B[3];
  for (int j = 0; j < 3; j++) A[j] = cmul(expfac, cadd(cscale(t1, p[j]), cscale(t2, rv[j])));
  const cplx e3 = cmul(expfac, t3);
  if (electric) {
    for (int j = 0; j < 3; j++) B[j] = cplx{e3.re * rxp[j] / Z, e3.im * rxp[j] / Z};
    for (int j = 0; j < 3; j++) {
      EH[j] = A[j];
      EH[3 + j] = B[j];
    }
  }
  else {
    for (int j = 0; j < 3; j++) B[j] = cplx{-e3.re * rxp[j] * Z, -e3.im * rxp[j] * Z};
    for (int j = 0; j < 3; j++) {
      EH[j] = B[j];
      EH[3 + j] = A[j];
    }
  }
}

// Hankel function of the first kind J_n(x) + i Y_n(x), n = 0, 1, 2
MGB_GRN cplx hankel(int n, double x) { return cplx{jn(n, x), yn(n, x)}; }

MGB_GRN void green2d(cplx EH[6], const double x[3], double freq, double eps, double mu, const double x0[3], int c0,
                     cplx f0) {
  double rv[2] = {x[0] - x0[0], x[1] - x0[1]};
  const double r = sqrt(rv[0] * rv[0] + rv[1] * rv[1]);
  rv[0] = rv[0] * (1.0 / r);
  rv[1] = rv[1] * (1.0 / r);
  const double omega = 2 * PI * freq;
  const double k = omega * sqrt(eps * mu);
  const double kr = k * r;
  const double Z = sqrt(mu / eps);
  const cplx H0 = cmul(hankel(0, kr), f0);
  const cplx H1 = cmul(hankel(1, kr), f0);
  // 0.25 * (i k) * H1
  const cplx ik = {0.0, k};
  const cplx q = cplx{0.25 * ik.re, 0.25 * ik.im};
  const cplx ikH1 = cmul(q, H1);
  const cplx zero = {0.0, 0.0};
  const int d = c0 % 3;
  const bool electric = c0 < 3;
  if (d == 2) {
    if (electric) {
      EH[0] = EH[1] = zero;
      EH[2] = cscale(H0, -0.25 * omega * mu);
      EH[3] = cscale(ikH1, -rv[1]);
      EH[4] = cscale(ikH1, rv[0]);
      EH[5] = zero;
    }
    else {
      EH[0] = cscale(ikH1, rv[1]);
      EH[1] = cscale(ikH1, -rv[0]);
      EH[2] = zero;
      EH[3] = EH[4] = zero;
      EH[5] = cscale(H0, -0.25 * omega * eps);
    }
    return;
  }
  const cplx H2 = cmul(hankel(2, kr), f0);
  const double p[2] = {d == 0 ? 1.0 : 0.0, d == 1 ? 1.0 : 0.0};
  const double pdotr = p[0] * rv[0] + p[1] * rv[1];
  const double rxp = rv[0] * p[1] - rv[1] * p[0];
  const cplx H02 = csub(H0, H2);
  if (electric) {
    const double a = pdotr / r * 0.25 * Z, b = rxp * omega * mu * 0.125;
    EH[0] = cadd(cscale(H1, -(rv[0] * a)), cscale(H02, rv[1] * b));
    EH[1] = csub(cscale(H1, -(rv[1] * a)), cscale(H02, rv[0] * b));
    EH[2] = zero;
    EH[3] = EH[4] = zero;
    EH[5] = cscale(ikH1, -rxp);
  }
  else {
    const double a = pdotr / r * 0.25 / Z, b = rxp * omega * eps * 0.125;
    EH[0] = EH[1] = zero;
    EH[2] = cscale(ikH1, rxp);
    EH[3] = cadd(cscale(H1, -(rv[0] * a)), cscale(H02, rv[1] * b));
    EH[4] = csub(cscale(H1, -(rv[1] * a)), cscale(H02, rv[0] * b));
    EH[5] = zero;
  }
}

} // namespace mgb_green

#endif
