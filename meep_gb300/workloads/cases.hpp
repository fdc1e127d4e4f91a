/* Synthetic FDTD workloads, written against the reference's C++ API
 * (meep.hpp), so the same code runs on the reference core and on this
 * repository's drop-in (include/meep_gb300/meep.hpp).  Used by the golden-
 * fixture driver (tests/golden/golden_driver.cpp) and the benchmark
 * (meep_gb300/workloads/bench_main.cpp).
 *
 * Geometry comes from std::mt19937_64 with fixed seeds.  The configurations
 * follow the benchmark definitions of this engine:
 *   tm2d   2-D TM, eps=12 cylinders in air, PML, Gaussian Ez point source,
 *          x-normal flux line (full size 512x512 cells, resolution 16, 40
 *          cylinders, 400-cell line, 51 frequencies, 4000 steps)
 *   vec3d  3-D, boxes of eps in {2.1, 4, 12}, 20% diagonally anisotropic,
 *          PML, Gaussian Ex dipole, z-normal flux plane (full size 256^3 at
 *          resolution 20, 200x200 plane, 50 frequencies, 1000 steps)
 *   disp3d 3-D, lower half Drude (1e-5, 0.05, sigma 50) + Lorentz (0.8, 0.1,
 *          sigma 2) poles, upper half D conductivity 0.01, line of Gaussian Ez
 *          sources, DFT of Ez on a full xy plane (full size 384x384x192,
 *          200 frequencies)
 */
#ifndef MEEP_GB300_WORKLOADS_CASES_HPP
#define MEEP_GB300_WORKLOADS_CASES_HPP

#include <meep.hpp>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <memory>
#include <random>
#include <vector>

namespace workloads {
using namespace meep;

/* --------------------------------------------------------------- geometry */
struct Cyl {
  double x, y, r;
};
struct Box {
  double lo[3], hi[3];
  double eps[3]; // diagonal entries (equal unless anisotropic)
};

class case_material : public material_function {
public:
  int dim = 2;
  double eps_bg = 1.0;
  std::vector<Cyl> cyls;
  double cyl_eps = 12.0;
  std::vector<Box> boxes;
  // dispersive / conductive layers split at z = split_z (3-D) or y (2-D)
  bool layered = false;
  double split = 0.0;
  double sigma_lower = 0.0; // susceptibility strength below the split
  double cond_upper = 0.0;  // D conductivity above the split

  // anisotropic boxes rotated by 30 degrees about z: chi1inv = R diag(1/eps) R^T
  // has xy off-diagonal entries (the structure then takes the two-pass
  // off-diagonal D/E update)
  bool rotate_aniso = false;

  double coord_split(const vec &r) const { return dim == 3 ? r.z() : r.y(); }

  void eps_diag(const vec &r, double e[3]) const {
    e[0] = e[1] = e[2] = eps_bg;
    for (const Cyl &c : cyls) {
      double dx = r.x() - c.x, dy = r.y() - c.y;
      if (dx * dx + dy * dy < c.r * c.r) e[0] = e[1] = e[2] = cyl_eps;
    }
    for (const Box &b : boxes) {
      bool in = true;
      for (int d = 0; d < dim; d++) {
        double v = d == 0 ? r.x() : (d == 1 ? r.y() : r.z());
        if (!(v > b.lo[d] && v < b.hi[d])) in = false;
      }
      if (in) {
        e[0] = b.eps[0];
        e[1] = b.eps[1];
        e[2] = b.eps[2];
      }
    }
  }
  virtual double chi1p1(field_type ft, const vec &r) {
    if (ft == H_stuff) return 1.0;
    double e[3];
    eps_diag(r, e);
    return e[0];
  }
  virtual void eff_chi1inv_row(component c, double row[3], const volume &v, double tol,
                               int maxeval) {
    (void)tol;
    (void)maxeval;
    row[0] = row[1] = row[2] = 0.0;
    double e[3];
    if (type(c) == H_stuff) {
      row[component_direction(c) % 3] = 1.0;
      return;
    }
    eps_diag(v.center(), e);
    const int d = component_direction(c) % 3;
    if (rotate_aniso && d < 2 && (e[0] != e[1])) {
      const double cs = std::sqrt(0.75), sn = 0.5;
      const double i0 = 1.0 / e[0], i1 = 1.0 / e[1];
      const double xx = cs * cs * i0 + sn * sn * i1, yy = sn * sn * i0 + cs * cs * i1, xy = cs * sn * (i0 - i1);
      row[0] = d == 0 ? xx : xy;
      row[1] = d == 0 ? xy : yy;
      return;
    }
    row[d] = 1.0 / e[d];
  }
  virtual bool is_thread_safe() const { return true; }
  virtual bool has_conductivity(component c) { return cond_upper != 0.0 && is_D(c); }
  virtual double conductivity(component c, const vec &r) {
    (void)c;
    return coord_split(r) > split ? cond_upper : 0.0;
  }
  virtual void sigma_row(component c, double row[3], const vec &r) {
    row[0] = row[1] = row[2] = 0.0;
    row[component_direction(c) % 3] = coord_split(r) < split ? sigma_lower : 0.0;
  }
};

/* A sigma function that is `scale` below the split and 0 above, for one pole. */
class pole_sigma : public material_function {
public:
  int dim;
  double split, scale;
  pole_sigma(int d, double s, double k) : dim(d), split(s), scale(k) {}
  virtual void sigma_row(component c, double row[3], const vec &r) {
    row[0] = row[1] = row[2] = 0.0;
    double v = dim == 3 ? r.z() : r.y();
    row[component_direction(c) % 3] = v < split ? scale : 0.0;
  }
};



inline std::vector<double> lin_space(double a, double b, int n) {
  std::vector<double> v(n);
  for (int i = 0; i < n; i++)
    v[i] = n > 1 ? a + (b - a) * i / (n - 1) : a;
  return v;
}

/* One configured simulation: structure, fields and monitors. */
struct Workload {
  grid_volume gv;
  case_material mat;
  std::unique_ptr<pole_sigma> drude, lorentz;
  std::unique_ptr<structure> s;
  std::unique_ptr<fields> f;
  std::unique_ptr<dft_flux> flux;
  std::unique_ptr<dft_fields> dftf;
  int nfreq = 0;
  double cells() const {
    double n = 1;
    LOOP_OVER_DIRECTIONS(gv.dim, d) n *= gv.num_direction(d);
    return n;
  }
};

inline std::unique_ptr<Workload> make_tm2d(int ncells_x, int ncells_y, double res, double dpml,
                                           int ncyl, uint64_t seed, int flux_cells, int nfreq,
                                           int decimation) {
  std::unique_ptr<Workload> w(new Workload);
  double sx = ncells_x / res, sy = ncells_y / res;
  w->gv = vol2d(sx, sy, res);
  w->gv.center_origin();
  w->mat.dim = 2;
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> ux(-sx / 2 + dpml, sx / 2 - dpml);
  std::uniform_real_distribution<double> uy(-sy / 2 + dpml, sy / 2 - dpml);
  std::uniform_real_distribution<double> ur(0.5, 2.0);
  for (int i = 0; i < ncyl; i++) {
    Cyl c;
    c.x = ux(rng);
    c.y = uy(rng);
    c.r = ur(rng) * (res >= 16 ? 1.0 : 0.25);
    w->mat.cyls.push_back(c);
  }
  w->s.reset(new structure(w->gv, w->mat, pml(dpml), identity(), 0, 0.5, false));
  w->f.reset(new fields(w->s.get()));
  w->f->use_real_fields();
  double fcen = 0.15, df = 0.1;
  gaussian_src_time src(fcen, df);
  w->f->add_point_source(Ez, src, vec(0.0, 0.0));
  double xf = 0.25 * sx;
  double half = 0.5 * flux_cells / res;
  volume fv(vec(xf, -half), vec(xf, half));
  w->flux.reset(new dft_flux(
      w->f->add_dft_flux(X, fv, fcen - df / 2, fcen + df / 2, nfreq, true, true, decimation)));
  w->nfreq = nfreq;
  return w;
}

inline std::unique_ptr<Workload> make_vec3d(int nx, int ny, int nz, double res, double dpml,
                                            int nbox, uint64_t seed, int flux_cells, int nfreq,
                                            bool rotate_aniso = false) {
  std::unique_ptr<Workload> w(new Workload);
  double sx = nx / res, sy = ny / res, sz = nz / res;
  w->gv = vol3d(sx, sy, sz, res);
  w->gv.center_origin();
  w->mat.dim = 3;
  w->mat.rotate_aniso = rotate_aniso;
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> u01(0.0, 1.0);
  const double choices[3] = {2.1, 4.0, 12.0};
  double L[3] = {sx, sy, sz};
  for (int i = 0; i < nbox; i++) {
    Box b;
    for (int d = 0; d < 3; d++) {
      double lo = -L[d] / 2 + dpml, hi = L[d] / 2 - dpml;
      double c = lo + (hi - lo) * u01(rng);
      double h = (0.05 + 0.2 * u01(rng)) * (hi - lo);
      b.lo[d] = c - h;
      b.hi[d] = c + h;
    }
    double e = choices[std::min(2, int(3 * u01(rng)))];
    b.eps[0] = b.eps[1] = b.eps[2] = e;
    if (u01(rng) < 0.2)
      for (int d = 0; d < 3; d++)
        b.eps[d] = 2.0 + 10.0 * u01(rng);
    w->mat.boxes.push_back(b);
  }
  w->s.reset(new structure(w->gv, w->mat, pml(dpml), identity(), 0, 0.5, false));
  w->f.reset(new fields(w->s.get()));
  w->f->use_real_fields();
  double fcen = 0.2, df = 0.2;
  gaussian_src_time src(fcen, df);
  w->f->add_point_source(Ex, src, vec(0.1 / res, -0.3 / res, -0.25 * sz));
  double half = 0.5 * flux_cells / res;
  volume fv(vec(-half, -half, 0.25 * sz), vec(half, half, 0.25 * sz));
  w->flux.reset(new dft_flux(w->f->add_dft_flux(Z, fv, fcen - df / 2, fcen + df / 2, nfreq)));
  w->nfreq = nfreq;
  return w;
}

inline std::unique_ptr<Workload> make_disp3d(int nx, int ny, int nz, double res, double dpml,
                                             int nfreq, int decimation) {
  std::unique_ptr<Workload> w(new Workload);
  double sx = nx / res, sy = ny / res, sz = nz / res;
  w->gv = vol3d(sx, sy, sz, res);
  w->gv.center_origin();
  w->mat.dim = 3;
  w->mat.layered = true;
  w->mat.split = 0.0;
  w->mat.cond_upper = 0.01;
  w->s.reset(new structure(w->gv, w->mat, pml(dpml), identity(), 0, 0.5, false));
  w->drude.reset(new pole_sigma(3, 0.0, 50.0));
  w->lorentz.reset(new pole_sigma(3, 0.0, 2.0));
  w->s->add_susceptibility(*w->drude, E_stuff, lorentzian_susceptibility(1e-5, 0.05, true));
  w->s->add_susceptibility(*w->lorentz, E_stuff, lorentzian_susceptibility(0.8, 0.1, false));
  w->f.reset(new fields(w->s.get()));
  w->f->use_real_fields();
  double fcen = 0.5, df = 0.6;
  gaussian_src_time src(fcen, df);
  double zs = 0.25 * sz;
  w->f->add_volume_source(Ez, src,
                          volume(vec(-0.5 * sx + dpml, 0.0, zs), vec(0.5 * sx - dpml, 0.0, zs)),
                          std::complex<double>(1.0, 0.0));
  component cz = Ez;
  double zm = -0.125 * sz;
  volume plane(vec(-0.5 * sx, -0.5 * sy, zm), vec(0.5 * sx, 0.5 * sy, zm));
  std::vector<double> freqs = lin_space(fcen - df / 2, fcen + df / 2, nfreq);
  w->dftf.reset(new dft_fields(
      w->f->add_dft_fields(&cz, 1, plane, freqs.data(), freqs.size(), true, decimation)));
  w->nfreq = nfreq;
  return w;
}

} // namespace workloads
#endif
