/* Golden-fixture driver for the FDTD stepping path.
 *
 * Written against the reference's C++ API (meep.hpp: structure, fields,
 * add_point_source/add_volume_source, add_dft_flux, add_dft_fields, step) so
 * that the SAME source builds three ways:
 *   - against the reference core (oracle/_ref, CPU, FP64 or FP32): the golden
 *     fixtures in tests/golden (.bin files) are its output;
 *   - against this repository's drop-in header include/meep_gb300/meep.hpp with
 *     the CUDA engine (product path, runs on the GPU);
 *   - against the same drop-in header with the CPU oracle backend (tests).
 *
 * Usage: golden_driver <case> <out.bin> [steps]
 * Output: a flat record file, each record = u32 name length, name bytes,
 * u64 count, count little-endian doubles (see tests/golden/records.py).
 *
 * Geometry is drawn from std::mt19937_64 with fixed seeds, so every build sees
 * the same structure. */
#include <meep.hpp>

#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <random>
#include <string>
#include <vector>

using namespace meep;
using std::complex;

#ifndef MEEP_GB300
// The reference keeps DFT sums in host memory already.
static void sync_dfts(fields &) {}
#endif

/* ----------------------------------------------------------------- output */
struct Writer {
  FILE *fp;
  explicit Writer(const char *path) {
    fp = fopen(path, "wb");
    if (!fp) {
      fprintf(stderr, "cannot open %s\n", path);
      exit(2);
    }
  }
  ~Writer() { fclose(fp); }
  void rec(const std::string &name, const std::vector<double> &v) {
    uint32_t n = (uint32_t)name.size();
    uint64_t c = v.size();
    fwrite(&n, 4, 1, fp);
    fwrite(name.data(), 1, n, fp);
    fwrite(&c, 8, 1, fp);
    if (c) fwrite(v.data(), 8, c, fp);
  }
  void scalar(const std::string &name, double x) { rec(name, std::vector<double>(1, x)); }
};

/* Global array of component c at every Yee point of the cell: for each
   direction of the grid, points k = 0..n with ivec coordinate io + shift + 2k
   (fastest index last: x, y, z order of the directions present). */
static std::vector<double> global_field(fields &f, const grid_volume &gv, component c) {
  std::vector<double> out;
  ivec io = gv.little_corner();
  ivec sh = gv.iyee_shift(c);
  int n[3] = {1, 1, 1};
  direction ds[3];
  int nd = 0;
  LOOP_OVER_DIRECTIONS(gv.dim, d) {
    ds[nd] = d;
    n[nd] = gv.num_direction(d) + 1;
    nd++;
  }
  for (int a = 0; a < n[0]; a++)
    for (int b = 0; b < (nd > 1 ? n[1] : 1); b++)
      for (int cc = 0; cc < (nd > 2 ? n[2] : 1); cc++) {
        ivec p = io + sh;
        int k[3] = {a, b, cc};
        for (int q = 0; q < nd; q++)
          p.set_direction(ds[q], p.in_direction(ds[q]) + 2 * k[q]);
        out.push_back(real(f.get_field(c, p, false)));
      }
  return out;
}

/* DFT chunk contents as (coordinates, values): for every point of every chunk
   of the monitor, the ivec coordinates followed by Re, Im at each frequency. */
static std::vector<double> dump_dft_chunks(dft_chunk *chunks, component c, const grid_volume &gv) {
  std::map<std::vector<int>, std::vector<double> > pts;
  for (dft_chunk *ch = chunks; ch; ch = ch->next_in_dft) {
    if (ch->c != c) continue;
    size_t nw = ch->omega.size();
    int lo[3] = {0, 0, 0}, cnt[3] = {1, 1, 1};
    int nd = 0;
    LOOP_OVER_DIRECTIONS(gv.dim, d) {
      lo[nd] = ch->is.in_direction(d);
      cnt[nd] = (ch->ie.in_direction(d) - ch->is.in_direction(d)) / 2 + 1;
      nd++;
    }
    size_t idx = 0;
    for (int a = 0; a < cnt[0]; a++)
      for (int b = 0; b < cnt[1]; b++)
        for (int e = 0; e < cnt[2]; e++, idx++) {
          std::vector<int> key;
          int k[3] = {a, b, e};
          for (int q = 0; q < nd; q++)
            key.push_back(lo[q] + 2 * k[q]);
          std::vector<double> vals;
          for (size_t w = 0; w < nw; w++) {
            vals.push_back(real(ch->dft[idx * nw + w]));
            vals.push_back(imag(ch->dft[idx * nw + w]));
          }
          pts[key] = vals;
        }
  }
  std::vector<double> out;
  for (auto &kv : pts) {
    for (int x : kv.first)
      out.push_back(x);
    for (double v : kv.second)
      out.push_back(v);
  }
  return out;
}

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
    row[component_direction(c) % 3] = 1.0 / e[component_direction(c) % 3];
  }
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

static std::vector<double> linspace(double a, double b, int n) {
  std::vector<double> v(n);
  for (int i = 0; i < n; i++)
    v[i] = n > 1 ? a + (b - a) * i / (n - 1) : a;
  return v;
}

/* ------------------------------------------------------------------ cases */

/* 2-D TM (Ez, Hx, Hy): cylinders of eps=12 in air, PML on all sides, Gaussian
   Ez point source at the centre, x-normal flux line.  The full-size variant is
   512x512 cells at resolution 16 with 40 cylinders, 4000 steps, a 400-cell
   flux line at 51 frequencies. */
static void case_tm2d(Writer &w, int ncells_x, int ncells_y, double res, double dpml, int ncyl,
                      uint64_t seed, int steps, int flux_cells, int nfreq, bool dump_fields,
                      int decimation) {
  double sx = ncells_x / res, sy = ncells_y / res;
  grid_volume gv = vol2d(sx, sy, res);
  gv.center_origin();
  case_material mat;
  mat.dim = 2;
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> ux(-sx / 2 + dpml, sx / 2 - dpml);
  std::uniform_real_distribution<double> uy(-sy / 2 + dpml, sy / 2 - dpml);
  std::uniform_real_distribution<double> ur(0.5, 2.0);
  for (int i = 0; i < ncyl; i++) {
    Cyl c;
    c.x = ux(rng);
    c.y = uy(rng);
    c.r = ur(rng) * (res >= 16 ? 1.0 : 0.25);
    mat.cyls.push_back(c);
  }
  structure s(gv, mat, pml(dpml), identity(), 0, 0.5, false);
  fields f(&s);
  f.use_real_fields();
  double fcen = 0.15, df = 0.1;
  gaussian_src_time src(fcen, df);
  f.add_point_source(Ez, src, vec(0.0, 0.0));
  double xf = 0.25 * sx;
  double half = 0.5 * flux_cells / res;
  volume fv(vec(xf, -half), vec(xf, half));
  dft_flux fl = f.add_dft_flux(X, fv, fcen - df / 2, fcen + df / 2, nfreq, true, true, decimation);
  for (int i = 0; i < steps; i++)
    f.step();
  sync_dfts(f);
  double *F = fl.flux();
  w.rec("flux", std::vector<double>(F, F + nfreq));
  delete[] F;
  w.scalar("t", f.time());
  if (dump_fields) {
    w.rec("Ez", global_field(f, gv, Ez));
    w.rec("Hx", global_field(f, gv, Hx));
    w.rec("Hy", global_field(f, gv, Hy));
    w.rec("dft_Ez", dump_dft_chunks(fl.E, Ez, gv));
    w.rec("dft_Hy", dump_dft_chunks(fl.H, Hy, gv));
  }
}

/* 3-D full-vector, non-dispersive: boxes of eps in {2.1, 4, 12}, 20% of them
   diagonally anisotropic, PML on all faces, Gaussian Ex dipole, z-normal flux
   plane. */
static void case_vec3d(Writer &w, int nx, int ny, int nz, double res, double dpml, int nbox,
                       uint64_t seed, int steps, int flux_cells, int nfreq, bool dump_fields) {
  double sx = nx / res, sy = ny / res, sz = nz / res;
  grid_volume gv = vol3d(sx, sy, sz, res);
  gv.center_origin();
  case_material mat;
  mat.dim = 3;
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
    mat.boxes.push_back(b);
  }
  structure s(gv, mat, pml(dpml), identity(), 0, 0.5, false);
  fields f(&s);
  f.use_real_fields();
  double fcen = 0.2, df = 0.2;
  gaussian_src_time src(fcen, df);
  f.add_point_source(Ex, src, vec(0.1 / res, -0.3 / res, -0.25 * sz));
  double half = 0.5 * flux_cells / res;
  volume fv(vec(-half, -half, 0.25 * sz), vec(half, half, 0.25 * sz));
  dft_flux fl = f.add_dft_flux(Z, fv, fcen - df / 2, fcen + df / 2, nfreq);
  for (int i = 0; i < steps; i++)
    f.step();
  sync_dfts(f);
  double *F = fl.flux();
  w.rec("flux", std::vector<double>(F, F + nfreq));
  delete[] F;
  w.scalar("t", f.time());
  if (dump_fields) {
    const component cs[6] = {Ex, Ey, Ez, Hx, Hy, Hz};
    const char *names[6] = {"Ex", "Ey", "Ez", "Hx", "Hy", "Hz"};
    for (int i = 0; i < 6; i++)
      w.rec(names[i], global_field(f, gv, cs[i]));
    w.rec("dft_Ex", dump_dft_chunks(fl.E, Ex, gv));
    w.rec("dft_Hy", dump_dft_chunks(fl.H, Hy, gv));
  }
}

/* 3-D dispersive: lower half (z < 0) is a Drude pole (omega 1e-5, gamma 0.05,
   sigma 50) plus a Lorentz pole (omega 0.8, gamma 0.1, sigma 2); the upper half
   has D conductivity 0.01.  A line of Gaussian Ez sources along x; DFT fields
   of Ez on a full xy plane. */
static void case_disp3d(Writer &w, int nx, int ny, int nz, double res, double dpml, int steps,
                        int nfreq, bool dump_fields, int decimation) {
  double sx = nx / res, sy = ny / res, sz = nz / res;
  grid_volume gv = vol3d(sx, sy, sz, res);
  gv.center_origin();
  case_material mat;
  mat.dim = 3;
  mat.layered = true;
  mat.split = 0.0;
  mat.cond_upper = 0.01;
  structure s(gv, mat, pml(dpml), identity(), 0, 0.5, false);
  pole_sigma drude(3, 0.0, 50.0), lorentz(3, 0.0, 2.0);
  s.add_susceptibility(drude, E_stuff, lorentzian_susceptibility(1e-5, 0.05, true));
  s.add_susceptibility(lorentz, E_stuff, lorentzian_susceptibility(0.8, 0.1, false));
  fields f(&s);
  f.use_real_fields();
  double fcen = 0.5, df = 0.6;
  gaussian_src_time src(fcen, df);
  double zs = 0.25 * sz;
  f.add_volume_source(Ez, src, volume(vec(-0.5 * sx + dpml, 0.0, zs), vec(0.5 * sx - dpml, 0.0, zs)),
                      complex<double>(1.0, 0.0));
  component cz = Ez;
  double zm = -0.125 * sz;
  volume plane(vec(-0.5 * sx, -0.5 * sy, zm), vec(0.5 * sx, 0.5 * sy, zm));
  std::vector<double> freqs = linspace(fcen - df / 2, fcen + df / 2, nfreq);
  dft_fields dfld = f.add_dft_fields(&cz, 1, plane, freqs.data(), freqs.size(), true, decimation);
  for (int i = 0; i < steps; i++)
    f.step();
  sync_dfts(f);
  w.scalar("t", f.time());
  w.rec("dft_Ez", dump_dft_chunks(dfld.chunks, Ez, gv));
  if (dump_fields) {
    w.rec("Ex", global_field(f, gv, Ex));
    w.rec("Ez", global_field(f, gv, Ez));
    w.rec("Hy", global_field(f, gv, Hy));
  }
}

/* Known answers from the reference's own test suite (tests/known_results.cpp)
   that lie on this path: 2-D TM metallic and PML, 3-D metallic, 1-D Lorentz
   polariton.  Same structures, sources and run lengths. */
static double one_eps(const vec &) { return 1.0; }
static double sigma_763(const vec &) { return 7.63; }

static void case_known(Writer &w) {
  const double a = 10.0;
  {
    grid_volume gv = voltwo(1.0, 1.0, a);
    structure s(gv, one_eps);
    fields f(&s);
    f.add_point_source(Ez, 0.2, 3.0, 0.0, 2.0, gv.center(), complex<double>(0, -2 * pi * 0.2));
    while (f.round_time() < 10.0)
      f.step();
    w.scalar("metallic_2d_tm", real(f.get_field(Ez, gv.center())));
  }
  {
    double dpml = 1.0;
    grid_volume gv = voltwo(1.0 + 2 * dpml, 1.0 + 2 * dpml, a);
    structure s(gv, one_eps, pml(dpml));
    fields f(&s);
    f.add_point_source(Ez, 0.2, 3.0, 0.0, 2.0, gv.center(), complex<double>(0, -2 * pi * 0.2));
    while (f.round_time() < 30.0)
      f.step();
    w.scalar("pml_2d_tm", real(f.get_field(Ez, gv.center())));
  }
  {
    grid_volume gv = vol3d(1.0, 1.0, 1.0, a);
    structure s(gv, one_eps);
    fields f(&s);
    f.add_point_source(Ez, 0.2, 3.0, 0.0, 2.0, gv.center(), complex<double>(0, -2 * pi * 0.2));
    while (f.round_time() < 10.0)
      f.step();
    w.scalar("metallic_3d", real(f.get_field(Ez, gv.center())));
  }
  {
    grid_volume gv = volone(1.0, a);
    structure s(gv, one_eps);
    s.add_susceptibility(sigma_763, E_stuff, lorentzian_susceptibility(0.3, 0.1));
    fields f(&s);
    f.add_point_source(Ex, 0.2, 3.0, 0.0, 2.0, gv.center(), complex<double>(0, -2 * pi * 0.2));
    while (f.round_time() < 10.0)
      f.step();
    w.scalar("polariton_1d", real(f.get_field(Ex, gv.center())));
  }
}

int main(int argc, char **argv) {
  initialize mpi(argc, argv);
  verbosity = 0;
  if (argc < 3) {
    fprintf(stderr, "usage: %s case out.bin [steps]\n", argv[0]);
    return 2;
  }
  std::string cs = argv[1];
  Writer w(argv[2]);
  int steps = argc > 3 ? atoi(argv[3]) : -1;
  w.scalar("realnum_bytes", (double)sizeof(realnum));
  if (cs == "tm2d_small")
    case_tm2d(w, 64, 48, 10.0, 1.0, 6, 1234, steps > 0 ? steps : 1600, 30, 11, true, 0);
  else if (cs == "tm2d_small_dec1")
    case_tm2d(w, 64, 48, 10.0, 1.0, 6, 1234, steps > 0 ? steps : 1600, 30, 11, true, 1);
  else if (cs == "tm2d_full")
    case_tm2d(w, 512, 512, 16.0, 1.0, 40, 1234, steps > 0 ? steps : 4000, 400, 51, false, 0);
  else if (cs == "vec3d_small")
    case_vec3d(w, 24, 20, 18, 20.0, 0.25, 6, 42, steps > 0 ? steps : 1200, 10, 9, true);
  else if (cs == "vec3d_full")
    case_vec3d(w, 256, 256, 256, 20.0, 0.8, 60, 42, steps > 0 ? steps : 1000, 200, 50, false);
  else if (cs == "disp3d_small")
    case_disp3d(w, 20, 18, 16, 20.0, 0.25, steps > 0 ? steps : 600, 7, true, 1);
  else if (cs == "known")
    case_known(w);
  else {
    fprintf(stderr, "unknown case %s\n", cs.c_str());
    return 2;
  }
  return 0;
}
