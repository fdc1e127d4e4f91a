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

#include "cases.hpp"

#include <algorithm>
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
#include "meep_internals.hpp" // src_vol, for the adjoint case's source points
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

/* ------------------------------------------------------------------ cases */
using namespace workloads;

static void run_steps(Workload &wl, int steps) {
  for (int i = 0; i < steps; i++)
    wl.f->step();
  sync_dfts(*wl.f);
}

static void write_flux(Writer &w, Workload &wl) {
  double *F = wl.flux->flux();
  w.rec("flux", std::vector<double>(F, F + wl.nfreq));
  delete[] F;
}

static void case_tm2d(Writer &w, int ncells_x, int ncells_y, double res, double dpml, int ncyl,
                      uint64_t seed, int steps, int flux_cells, int nfreq, bool dump_fields,
                      int decimation) {
  auto wl = make_tm2d(ncells_x, ncells_y, res, dpml, ncyl, seed, flux_cells, nfreq, decimation);
  run_steps(*wl, steps);
  write_flux(w, *wl);
  w.scalar("t", wl->f->time());
  if (dump_fields) {
    w.rec("Ez", global_field(*wl->f, wl->gv, Ez));
    w.rec("Hx", global_field(*wl->f, wl->gv, Hx));
    w.rec("Hy", global_field(*wl->f, wl->gv, Hy));
    w.rec("dft_Ez", dump_dft_chunks(wl->flux->E, Ez, wl->gv));
    w.rec("dft_Hy", dump_dft_chunks(wl->flux->H, Hy, wl->gv));
  }
}

static void case_vec3d(Writer &w, int nx, int ny, int nz, double res, double dpml, int nbox,
                       uint64_t seed, int steps, int flux_cells, int nfreq, bool dump_fields) {
  auto wl = make_vec3d(nx, ny, nz, res, dpml, nbox, seed, flux_cells, nfreq);
  run_steps(*wl, steps);
  write_flux(w, *wl);
  w.scalar("t", wl->f->time());
  if (dump_fields) {
    const component cs[6] = {Ex, Ey, Ez, Hx, Hy, Hz};
    const char *names[6] = {"Ex", "Ey", "Ez", "Hx", "Hy", "Hz"};
    for (int i = 0; i < 6; i++)
      w.rec(names[i], global_field(*wl->f, wl->gv, cs[i]));
    w.rec("dft_Ex", dump_dft_chunks(wl->flux->E, Ex, wl->gv));
    w.rec("dft_Hy", dump_dft_chunks(wl->flux->H, Hy, wl->gv));
  }
}

static void case_disp3d(Writer &w, int nx, int ny, int nz, double res, double dpml, int steps,
                        int nfreq, bool dump_fields, int decimation) {
  auto wl = make_disp3d(nx, ny, nz, res, dpml, nfreq, decimation);
  run_steps(*wl, steps);
  w.scalar("t", wl->f->time());
  w.rec("dft_Ez", dump_dft_chunks(wl->dftf->chunks, Ez, wl->gv));
  if (dump_fields) {
    w.rec("Ex", global_field(*wl->f, wl->gv, Ex));
    w.rec("Ez", global_field(*wl->f, wl->gv, Ez));
    w.rec("Hy", global_field(*wl->f, wl->gv, Hy));
  }
}

/* One z plane (point index kz along z) of component c: every `every`-th of
   the (nx+1)(ny+1) points of its own Yee grid in x-slowest order. */
static std::vector<double> plane_field(fields &f, const grid_volume &gv, component c, int kz, int every = 7) {
  std::vector<double> out;
  ivec p0 = gv.little_corner() + gv.iyee_shift(c);
  long long n = 0;
  for (int a = 0; a <= gv.nx(); a++)
    for (int b = 0; b <= gv.ny(); b++) {
      if (n++ % every) continue;
      ivec p = p0;
      p.set_direction(X, p0.in_direction(X) + 2 * a);
      p.set_direction(Y, p0.in_direction(Y) + 2 * b);
      p.set_direction(Z, p0.in_direction(Z) + 2 * kz);
      out.push_back(real(f.get_field(c, p, false)));
    }
  return out;
}

/* Large DFT monitors in a few numbers: per frequency the sum of |F|^2 over
   every point and the projection sum_k r_k F_k onto signs r_k = +-1 drawn
   from a hash of the point's ivec coordinates (both complex sums, order
   independent to rounding); plus the full spectra of every point whose
   coordinates hash into one residue class mod `every` (coordinates, then
   Re, Im per frequency). */
static uint64_t coord_hash(const ivec &p) {
  uint64_t h = 1469598103934665603ull;
  LOOP_OVER_DIRECTIONS(p.dim, d) {
    h ^= (uint64_t)(uint32_t)(p.in_direction(d) + 100000);
    h *= 1099511628211ull;
  }
  return h ^ (h >> 29);
}
static void write_dft_summary(Writer &w, const std::string &name, dft_chunk *chunks, component c,
                              const grid_volume &gv, int every) {
  std::vector<double> norm2, proj, sample;
  size_t nw = 0;
  for (dft_chunk *ch = chunks; ch; ch = ch->next_in_dft) {
    if (ch->c != c) continue;
    nw = ch->omega.size();
    if (norm2.empty()) {
      norm2.assign(nw, 0.0);
      proj.assign(2 * nw, 0.0);
    }
    int cnt[3] = {1, 1, 1};
    direction ds[3];
    int nd = 0;
    LOOP_OVER_DIRECTIONS(gv.dim, d) {
      ds[nd] = d;
      cnt[nd] = (ch->ie.in_direction(d) - ch->is.in_direction(d)) / 2 + 1;
      nd++;
    }
    size_t idx = 0;
    for (int a = 0; a < cnt[0]; a++)
      for (int b = 0; b < cnt[1]; b++)
        for (int e = 0; e < cnt[2]; e++, idx++) {
          ivec p = ch->is;
          int k[3] = {a, b, e};
          for (int q = 0; q < nd; q++)
            p.set_direction(ds[q], ch->is.in_direction(ds[q]) + 2 * k[q]);
          const uint64_t h = coord_hash(p);
          const double r = (h & 1) ? 1.0 : -1.0;
          const bool keep = (h >> 1) % (uint64_t)every == 0;
          if (keep)
            for (int q = 0; q < nd; q++)
              sample.push_back(p.in_direction(ds[q]));
          for (size_t q = 0; q < nw; q++) {
            const complex<double> v(ch->dft[idx * nw + q]);
            norm2[q] += std::norm(v);
            proj[2 * q] += r * v.real();
            proj[2 * q + 1] += r * v.imag();
            if (keep) {
              sample.push_back(v.real());
              sample.push_back(v.imag());
            }
          }
        }
  }
  w.rec(name + "_norm2", norm2);
  w.rec(name + "_proj", proj);
  w.rec(name + "_sample", sample);
}

/* The benchmark workloads at full size, a few hundred steps (until the
   pulse has crossed the monitors): the 256^3 non-dispersive case (flux
   spectrum from 10 decimated samples, field planes at the flux plane, the
   grid centre and inside the low z PML) and the 384 x 384 x 192 dispersive
   case (six full 64-step blocks of the 200-frequency DFT of Ez on the whole
   plane, field planes at the DFT plane, the source plane and inside the low
   z PML).  Planes are every 7th point, DFT spectra a hashed sample. */
static void case_vec3d_full_trunc(Writer &w, int steps) {
  auto wl = make_vec3d(256, 256, 256, 20.0, 0.8, 60, 42, 200, 50);
  run_steps(*wl, steps);
  write_flux(w, *wl);
  w.scalar("t", wl->f->time());
  const component cs[4] = {Ex, Ey, Hx, Hz};
  const char *names[4] = {"Ex", "Ey", "Hx", "Hz"};
  const int planes[3] = {192, 128, 6};
  for (int i = 0; i < 4; i++)
    for (int kz : planes)
      w.rec(std::string(names[i]) + "_z" + std::to_string(kz), plane_field(*wl->f, wl->gv, cs[i], kz));
}

/* The dispersive workload on a 96^3 grid over its full 3000 steps: the
   single-precision error of the DFT spectrum, per frequency, is a property
   of the arithmetic; this case measures it for the reference's own FP32
   build.  Records: the DFT summary (a hashed sample of every 97th point);
   with GOLDEN_DFT_DUMP set, every point's spectrum is also written there as
   raw complex doubles (chunk order, frequency fastest). */
static void case_disp3d_cube(Writer &w, int steps) {
  auto wl = make_disp3d(96, 96, 96, 20.0, 0.8, 200, 1);
  run_steps(*wl, steps);
  w.scalar("t", wl->f->time());
  write_dft_summary(w, "dft_Ez", wl->dftf->chunks, Ez, wl->gv, 97);
  if (const char *path = getenv("GOLDEN_DFT_DUMP")) {
    FILE *fp = fopen(path, "wb");
    if (!fp) {
      fprintf(stderr, "cannot open %s\n", path);
      exit(2);
    }
    for (dft_chunk *ch = wl->dftf->chunks; ch; ch = ch->next_in_dft)
      for (size_t k = 0; k < ch->N * ch->omega.size(); k++) {
        const complex<double> v(ch->dft[k]);
        fwrite(&v, sizeof(v), 1, fp);
      }
    fclose(fp);
  }
}

static void case_disp3d_full_trunc(Writer &w, int steps) {
  auto wl = make_disp3d(384, 384, 192, 20.0, 0.8, 200, 1);
  run_steps(*wl, steps);
  w.scalar("t", wl->f->time());
  write_dft_summary(w, "dft_Ez", wl->dftf->chunks, Ez, wl->gv, 1999);
  const component cs[3] = {Ex, Ez, Hy};
  const char *names[3] = {"Ex", "Ez", "Hy"};
  const int planes[3] = {72, 144, 6};
  for (int i = 0; i < 3; i++)
    for (int kz : planes)
      w.rec(std::string(names[i]) + "_z" + std::to_string(kz), plane_field(*wl->f, wl->gv, cs[i], kz));
}

/* Known answers from the reference's own test suite (tests/known_results.cpp)
   that lie on this path: 2-D TM metallic and PML, 3-D metallic, 1-D Lorentz
   polariton.  Same structures, sources and run lengths. */
static double one_eps(const vec &) { return 1.0; }
static double sigma_763(const vec &) { return 7.63; }
// rods of eps 12 on a unit lattice (tests/known_results.cpp:28-41)
static double rods_eps(const vec &r) {
  vec p = r;
  while (p.x() < -0.5)
    p.set_direction(X, p.x() + 1.0);
  while (p.x() > 0.5)
    p.set_direction(X, p.x() - 1.0);
  while (p.y() < -0.5)
    p.set_direction(Y, p.y() + 1.0);
  while (p.y() > 0.5)
    p.set_direction(Y, p.y() - 1.0);
  if (p.x() * p.x() + p.y() * p.y() < 0.3) return 12.0;
  return 1.0;
}

// Bloch-periodic known results (tests/known_results.cpp:63-101): the same
// structures, sources, wavevectors and run lengths
static double known_x_periodic(const grid_volume &gv, double eps(const vec &), bool ypml) {
  structure s(gv, eps, ypml ? pml(1.0, Y) : boundary_region());
  fields f(&s);
  f.add_point_source(Ez, 0.2, 3.0, 0.0, 2.0, gv.center(), complex<double>(0, -2 * pi * 0.2));
  f.use_bloch(X, 0.1);
  while (f.round_time() < 30.0)
    f.step();
  return real(f.get_field(Ez, gv.center()));
}

static double known_periodic(const grid_volume &gv, double eps(const vec &)) {
  structure s(gv, eps);
  fields f(&s);
  f.add_point_source(Ez, 0.2, 3.0, 0.0, 2.0, gv.center(), complex<double>(0, -2 * pi * 0.2));
  vec k = gv.dim == D2 ? vec(0.3, 0.4) : vec(0.3, 0.5, 0.8);
  f.use_bloch(k);
  while (f.round_time() < 30.0)
    f.step();
  return real(f.get_field(Ez, gv.center()));
}

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
  w.scalar("x_periodic_2d", known_x_periodic(voltwo(1.0, 1.0, a), one_eps, false));
  w.scalar("periodic_2d_rods", known_periodic(voltwo(1.0, 3.0, a), rods_eps));
  w.scalar("periodic_2d", known_periodic(voltwo(1.0, 3.0, a), one_eps));
  w.scalar("x_periodic_y_pml_2d", known_x_periodic(voltwo(1.0, 3.0, a), one_eps, true));
  w.scalar("x_periodic_3d", known_x_periodic(vol3d(1.0, 1.0, 1.0, a), one_eps, false));
  w.scalar("x_periodic_y_pml_3d", known_x_periodic(vol3d(1.0, 3.0, 1.0, a), one_eps, true));
  w.scalar("periodic_3d_rods", known_periodic(vol3d(1.0, 1.0, 1.0, a), rods_eps));
  w.scalar("periodic_3d", known_periodic(vol3d(1.0, 1.0, 1.0, a), one_eps));
}

/* Scripts of the reference's Python interface, restated as the C++ calls its
   Python layer makes (python/simulation.py: _create_grid_volume +
   center_origin, PML boundary_region, geometry as a material_function with
   the last containing object winning, one polarization per distinct
   susceptibility, Source.add_source -> add_volume_source with
   gaussian_src_time(f, w, start, start + 2 w cutoff) and is_integrated,
   _add_fluxish_stuff -> add_dft_flux(volume_list prepended per region),
   add_dft_fields, _run_until / _run_sources_until stopping on round_time).
   tests/test_simulation_api.py runs the same scripts through the package's
   Simulation class. */
struct PyObj {
  int kind; // 0 block, 1 sphere, 2 cylinder (axis z, infinite height)
  double c[3], s[3], r;
  int mat;
};
struct PyMed {
  double eps[3], cond;
  double sig[2]; // sigma of susceptibility 0 and 1
};
class PyGeom : public material_function {
public:
  int dim = 2;
  std::vector<PyObj> objs;
  std::vector<PyMed> meds;
  const PyMed &at(const vec &r) const {
    double p[3] = {r.x(), r.y(), dim == 3 ? r.z() : 0.0};
    for (size_t q = objs.size(); q-- > 0;) {
      const PyObj &o = objs[q];
      double d[3] = {p[0] - o.c[0], p[1] - o.c[1], p[2] - o.c[2]};
      bool in;
      if (o.kind == 0) in = std::fabs(d[0]) <= 0.5 * o.s[0] && std::fabs(d[1]) <= 0.5 * o.s[1] &&
                            std::fabs(d[2]) <= 0.5 * o.s[2];
      else if (o.kind == 1) in = d[0] * d[0] + d[1] * d[1] + d[2] * d[2] <= o.r * o.r;
      else in = d[0] * d[0] + d[1] * d[1] <= o.r * o.r;
      if (in) return meds[o.mat];
    }
    return meds[0];
  }
  virtual double chi1p1(field_type ft, const vec &r) { return ft == H_stuff ? 1.0 : at(r).eps[0]; }
  virtual void eff_chi1inv_row(component c, double row[3], const volume &v, double, int) {
    row[0] = row[1] = row[2] = 0.0;
    int d = component_direction(c) % 3;
    row[d] = type(c) == H_stuff ? 1.0 : 1.0 / at(v.center()).eps[d];
  }
  virtual bool has_conductivity(component c) {
    if (!is_D(c)) return false;
    for (const PyMed &m : meds)
      if (m.cond != 0) return true;
    return false;
  }
  virtual double conductivity(component c, const vec &r) { return is_D(c) ? at(r).cond : 0.0; }
};
class PySigma : public material_function {
public:
  const PyGeom *g;
  int q;
  PySigma(const PyGeom *geo, int k) : g(geo), q(k) {}
  virtual void sigma_row(component c, double row[3], const vec &r) {
    row[0] = row[1] = row[2] = 0.0;
    row[component_direction(c) % 3] = g->at(r).sig[q];
  }
};

// numpy.linspace(a, b, n): a + i * ((b - a) / (n - 1)), last element b
static std::vector<double> np_linspace(double a, double b, int n) {
  std::vector<double> v(n);
  double step = (b - a) / (n - 1);
  for (int i = 0; i < n; i++)
    v[i] = i * step + a;
  v[n - 1] = b;
  return v;
}

static void py_run_until(fields &f, double until) {
  double t0 = f.round_time();
  while (!(f.round_time() >= t0 + until))
    f.step();
}

static void py_run_until_after_sources(fields &f, double T) {
  double ts = f.last_source_time();
  py_run_until(f, (ts - f.round_time()) + T);
}

/* Script:
     geometry = [mp.Block(mp.Vector3(mp.inf, 1, mp.inf), material=mp.Medium(epsilon=12)),
                 mp.Cylinder(0.8, center=mp.Vector3(3, 1.5), material=mp.Medium(index=2)),
                 mp.Sphere(0.6, center=mp.Vector3(-2, -1.7),
                           material=mp.Medium(epsilon=6, D_conductivity=0.05))]
     sim = mp.Simulation(cell_size=mp.Vector3(16, 8), resolution=10, geometry=geometry,
                         boundary_layers=[mp.PML(1.0)], eps_averaging=False,
                         sources=[mp.Source(mp.GaussianSource(0.15, fwidth=0.1), component=mp.Ez,
                                            center=mp.Vector3(-6), size=mp.Vector3(y=1))])
     tran = sim.add_flux([0.1, 0.125, 0.15, 0.175, 0.2],
                         mp.FluxRegion(center=mp.Vector3(6), size=mp.Vector3(y=2)))
     box = sim.add_flux(0.15, 0.05, 3, mp.FluxRegion(center=mp.Vector3(4), size=mp.Vector3(y=3)),
                        mp.FluxRegion(center=mp.Vector3(2), size=mp.Vector3(y=3), weight=-1))
     dft = sim.add_dft_fields([mp.Ez], [0.12, 0.15], center=mp.Vector3(5), size=mp.Vector3(1, 2))
     sim.run(until_after_sources=30) */
static void case_py_tm2d(Writer &w) {
  const double inf = 1.0e20;
  grid_volume gv = vol2d(16, 8, 10);
  gv.center_origin();
  PyGeom g;
  g.dim = 2;
  g.meds = {{{1, 1, 1}, 0, {0, 0}}, {{12, 12, 12}, 0, {0, 0}}, {{4, 4, 4}, 0, {0, 0}}, {{6, 6, 6}, 0.05, {0, 0}}};
  g.objs = {{0, {0, 0, 0}, {inf, 1, inf}, 0, 1}, {2, {3, 1.5, 0}, {0, 0, 0}, 0.8, 2},
            {1, {-2, -1.7, 0}, {0, 0, 0}, 0.6, 3}};
  structure s(gv, g, pml(1.0), identity(), 0, 0.5, false);
  fields f(&s);
  f.use_real_fields();
  double width = std::max(0.0, 1 / 0.1);
  gaussian_src_time src(0.15, width, 0.0, 0.0 + 2 * width * 5.0);
  src.is_integrated = false;
  f.add_volume_source(Ez, src, volume(vec(-6, -0.5), vec(-6, 0.5)), complex<double>(1.0, 0.0));
  std::vector<double> fr1 = {0.1, 0.125, 0.15, 0.175, 0.2};
  volume_list r1(volume(vec(6, -1), vec(6, 1)), Sx, 1.0);
  dft_flux tran = f.add_dft_flux(&r1, fr1.data(), fr1.size(), true, true, 0);
  std::vector<double> fr2 = np_linspace(0.15 - 0.5 * 0.05, 0.15 + 0.5 * 0.05, 3);
  volume_list *b1 = new volume_list(volume(vec(4, -1.5), vec(4, 1.5)), Sx, 1.0, nullptr);
  volume_list b2(volume(vec(2, -1.5), vec(2, 1.5)), Sx, -1.0, b1);
  dft_flux box = f.add_dft_flux(&b2, fr2.data(), fr2.size(), true, true, 0);
  component cs[1] = {Ez};
  std::vector<double> fr3 = {0.12, 0.15};
  dft_fields dft = f.add_dft_fields(cs, 1, volume(vec(4.5, -1), vec(5.5, 1)), fr3.data(), fr3.size(), true, 0);
  py_run_until_after_sources(f, 30);
  sync_dfts(f);
  double *F = tran.flux();
  w.rec("flux_tran", std::vector<double>(F, F + fr1.size()));
  delete[] F;
  F = box.flux();
  w.rec("flux_box", std::vector<double>(F, F + fr2.size()));
  delete[] F;
  w.scalar("t", f.time());
  w.rec("Ez", global_field(f, gv, Ez));
  w.rec("Hy", global_field(f, gv, Hy));
  w.rec("dft_Ez", dump_dft_chunks(dft.chunks, Ez, gv));
}

/* Script:
     mat = mp.Medium(epsilon=2, E_susceptibilities=[
         mp.LorentzianSusceptibility(frequency=1.1, gamma=0.1, sigma=0.5),
         mp.DrudeSusceptibility(frequency=0.8, gamma=0.05, sigma=0.3)])
     geometry = [mp.Block(mp.Vector3(1.2, 1.2, 1.2), material=mat),
                 mp.Sphere(0.4, center=mp.Vector3(0.6), material=mp.Medium(epsilon_diag=mp.Vector3(2, 3, 4)))]
     sim = mp.Simulation(cell_size=mp.Vector3(3, 3, 3), resolution=10, geometry=geometry,
                         boundary_layers=[mp.PML(0.5)], eps_averaging=False,
                         sources=[mp.Source(mp.GaussianSource(0.8, fwidth=0.5, is_integrated=True),
                                            component=mp.Ex, center=mp.Vector3(-0.7, 0.1))])
     flux = sim.add_flux(0.8, 0.4, 4, mp.FluxRegion(center=mp.Vector3(z=0.9), size=mp.Vector3(2, 2)))
     sim.run(until=8) */
static void case_py_disp3d(Writer &w) {
  grid_volume gv = vol3d(3, 3, 3, 10);
  gv.center_origin();
  PyGeom g;
  g.dim = 3;
  g.meds = {{{1, 1, 1}, 0, {0, 0}}, {{2, 2, 2}, 0, {0.5, 0.3}}, {{2, 3, 4}, 0, {0, 0}}};
  g.objs = {{0, {0, 0, 0}, {1.2, 1.2, 1.2}, 0, 1}, {1, {0.6, 0, 0}, {0, 0, 0}, 0.4, 2}};
  structure s(gv, g, pml(0.5), identity(), 0, 0.5, false);
  PySigma s0(&g, 0), s1(&g, 1);
  s.add_susceptibility(s0, E_stuff, lorentzian_susceptibility(1.1, 0.1));
  s.add_susceptibility(s1, E_stuff, lorentzian_susceptibility(0.8, 0.05, true));
  fields f(&s);
  f.use_real_fields();
  double width = std::max(0.0, 1 / 0.5);
  gaussian_src_time src(0.8, width, 0.0, 0.0 + 2 * width * 5.0);
  src.is_integrated = true;
  f.add_volume_source(Ex, src, volume(vec(-0.7, 0.1, 0), vec(-0.7, 0.1, 0)), complex<double>(1.0, 0.0));
  std::vector<double> fr = np_linspace(0.8 - 0.5 * 0.4, 0.8 + 0.5 * 0.4, 4);
  volume_list r(volume(vec(-1, -1, 0.9), vec(1, 1, 0.9)), Sz, 1.0);
  dft_flux flux = f.add_dft_flux(&r, fr.data(), fr.size(), true, true, 0);
  py_run_until(f, 8);
  double *F = flux.flux();
  w.rec("flux", std::vector<double>(F, F + fr.size()));
  delete[] F;
  w.scalar("t", f.time());
  w.rec("Ex", global_field(f, gv, Ex));
  w.rec("Hy", global_field(f, gv, Hy));
}

/* ------------------------------------------ subpixel averaging, off-diagonal
   Inverse-permittivity tensors with off-diagonal entries, from the default
   subpixel averaging of scalar material functions (structure(...,
   use_anisotropic_averaging = true), src/anisotropic_averaging.cpp) and from a
   material that supplies them itself (as tests/pml.cpp's offdiag_material
   does): the E update with OFFDIAG terms (src/step_generic.cpp:566-785),
   inside PML, with polarizations and integrated sources (f_minus_p), and with
   Bloch phases. */

// chi1inv entry (c, d) at every Yee point of c (0 where the cell does not own
// the point), same ordering as global_field
static std::vector<double> global_chi1inv(structure &s, const grid_volume &gv, component c, direction dd) {
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
        out.push_back(real(s.get_chi1inv(c, dd, p, 0, false)));
      }
  return out;
}

static std::vector<double> global_field_im(fields &f, const grid_volume &gv, component c) {
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
        out.push_back(imag(f.get_field(c, p, false)));
      }
  return out;
}

// a disk and a slab tilted against the grid: interface normals in every
// direction of the plane
static double lens_eps2d(const vec &r) {
  const double x = r.x(), y = r.y();
  const double dx = x + 0.7, dy = y - 0.3;
  if (dx * dx + dy * dy < 0.36) return 9.0;
  if (x > 0 && std::fabs(0.6 * x + 0.8 * y - 0.4) < 0.25) return 4.0;
  return 1.0;
}
static double lens_sigma2d(const vec &r) {
  const double dx = r.x() + 0.7, dy = r.y() - 0.3;
  return dx * dx + dy * dy < 0.36 ? 0.4 : 0.0;
}
static double lens_cond2d(const vec &r) {
  return r.x() > 0 && std::fabs(0.6 * r.x() + 0.8 * r.y() - 0.4) < 0.25 ? 0.05 : 0.0;
}

// 2-D TE (Ex, Ey, Hz) through the averaged lens: PML, a Lorentzian in the
// disk, D conductivity in the slab, an integrated Ey and a current Hz source
static void case_aniso_te2d(Writer &w, int steps) {
  grid_volume gv = vol2d(5.0, 4.0, 10.0);
  gv.center_origin();
  structure s(gv, lens_eps2d, pml(1.0), identity(), 0, 0.5, true);
  s.set_conductivity(Dx, lens_cond2d);
  s.set_conductivity(Dy, lens_cond2d);
  s.add_susceptibility(lens_sigma2d, E_stuff, lorentzian_susceptibility(1.2, 0.1));
  fields f(&s);
  f.use_real_fields();
  gaussian_src_time se(0.9, 0.6), sh(0.7, 0.5);
  f.add_point_source(Ey, se, vec(0.3, -0.6));
  sh.is_integrated = false;
  f.add_point_source(Hz, sh, vec(-1.2, 1.0), complex<double>(0.5, 0.0));
  std::vector<double> fr = {0.6, 0.75, 0.9, 1.05};
  volume_list r(volume(vec(1.4, -1.2), vec(1.4, 1.2)), Sx, 1.0);
  dft_flux flux = f.add_dft_flux(&r, fr.data(), fr.size(), true, true, 1);
  for (int i = 0; i < steps; i++)
    f.step();
  sync_dfts(f);
  double *F = flux.flux();
  w.rec("flux", std::vector<double>(F, F + fr.size()));
  delete[] F;
  w.scalar("t", f.time());
  w.rec("Ex", global_field(f, gv, Ex));
  w.rec("Ey", global_field(f, gv, Ey));
  w.rec("Hz", global_field(f, gv, Hz));
  w.rec("chi_ExX", global_chi1inv(s, gv, Ex, X));
  w.rec("chi_ExY", global_chi1inv(s, gv, Ex, Y));
  w.rec("chi_EyX", global_chi1inv(s, gv, Ey, X));
  w.rec("chi_EyY", global_chi1inv(s, gv, Ey, Y));
}

// a sphere and a slab whose normal is along no axis: full 3x3 tensors
static double lens_eps3d(const vec &r) {
  const double dx = r.x() - 0.1, dy = r.y() + 0.05, dz = r.z() - 0.05;
  if (dx * dx + dy * dy + dz * dz < 0.2025) return 6.0;
  if (std::fabs(0.48 * r.x() + 0.6 * r.y() + 0.64 * r.z() + 0.45) < 0.2) return 3.0;
  return 1.0;
}
static double lens_sigma3d(const vec &r) {
  const double dx = r.x() - 0.1, dy = r.y() + 0.05, dz = r.z() - 0.05;
  return dx * dx + dy * dy + dz * dz < 0.2025 ? 0.3 : 0.0;
}

static void case_aniso3d(Writer &w, int steps) {
  grid_volume gv = vol3d(1.8, 1.8, 1.8, 10.0);
  gv.center_origin();
  structure s(gv, lens_eps3d, pml(0.4), identity(), 0, 0.5, true);
  s.add_susceptibility(lens_sigma3d, E_stuff, lorentzian_susceptibility(1.0, 0.1));
  fields f(&s);
  f.use_real_fields();
  gaussian_src_time se(0.8, 0.6);
  f.add_point_source(Ex, se, vec(-0.3, 0.2, -0.1));
  f.add_point_source(Ez, se, vec(0.25, -0.3, 0.2), complex<double>(0.7, 0.0));
  std::vector<double> fr = {0.7, 0.8, 0.9};
  volume_list r(volume(vec(-0.4, -0.4, 0.45), vec(0.4, 0.4, 0.45)), Sz, 1.0);
  dft_flux flux = f.add_dft_flux(&r, fr.data(), fr.size(), true, true, 1);
  for (int i = 0; i < steps; i++)
    f.step();
  sync_dfts(f);
  double *F = flux.flux();
  w.rec("flux", std::vector<double>(F, F + fr.size()));
  delete[] F;
  w.scalar("t", f.time());
  const component cs[6] = {Ex, Ey, Ez, Hx, Hy, Hz};
  const char *names[6] = {"Ex", "Ey", "Ez", "Hx", "Hy", "Hz"};
  for (int i = 0; i < 6; i++)
    w.rec(names[i], global_field(f, gv, cs[i]));
  const char *dn[3] = {"X", "Y", "Z"};
  for (int c = 0; c < 3; c++)
    for (int d = 0; d < 3; d++)
      w.rec(std::string("chi_") + names[c] + dn[d], global_chi1inv(s, gv, cs[c], direction(d)));
}

// a material with a constant xy off-diagonal tensor everywhere, PML included
// (the tensor of tests/pml.cpp's offdiag_material, mu = 1)
class xy_offdiag_material : public material_function {
public:
  double od;
  explicit xy_offdiag_material(double o) : od(o) {}
  virtual void eff_chi1inv_row(component c, double row[3], const volume &v, double tol, int maxeval) {
    (void)v;
    (void)tol;
    (void)maxeval;
    const double detinv = 1.0 / (1 + 2 * od);
    row[0] = row[1] = row[2] = 0.0;
    if (type(c) != E_stuff) {
      row[component_direction(c) % 3] = 1.0;
      return;
    }
    if (component_direction(c) == X) {
      row[0] = (1 + od) * detinv;
      row[1] = -od * detinv;
    }
    else if (component_direction(c) == Y) {
      row[0] = -od * detinv;
      row[1] = (1 + od) * detinv;
    }
    else
      row[2] = 1.0;
  }
};

static double unit_cond(const vec &) { return 0.3; }

static void case_offdiag_te2d(Writer &w, int steps) {
  grid_volume gv = vol2d(4.0, 4.0, 10.0);
  gv.center_origin();
  structure s(gv, one_eps, pml(1.0), identity(), 0, 0.5, false);
  s.set_conductivity(Bz, unit_cond);
  xy_offdiag_material mat(0.5);
  s.set_materials(mat, false);
  fields f(&s);
  f.use_real_fields();
  gaussian_src_time src(1.0, 0.5);
  src.is_integrated = false;
  f.add_point_source(Hz, src, gv.center() + vec(0.25, -0.15));
  for (int i = 0; i < steps; i++)
    f.step();
  w.scalar("t", f.time());
  w.rec("Ex", global_field(f, gv, Ex));
  w.rec("Ey", global_field(f, gv, Ey));
  w.rec("Hz", global_field(f, gv, Hz));
}

// periodic lattice of disks with a Bloch wavevector: complex fields whose
// off-diagonal terms read D and P on the ghost planes
static double disk_eps(const vec &r) {
  vec p = r;
  while (p.x() < -0.5)
    p.set_direction(X, p.x() + 1.0);
  while (p.x() > 0.5)
    p.set_direction(X, p.x() - 1.0);
  while (p.y() < -0.5)
    p.set_direction(Y, p.y() + 1.0);
  while (p.y() > 0.5)
    p.set_direction(Y, p.y() - 1.0);
  return p.x() * p.x() + p.y() * p.y() < 0.1 ? 8.0 : 1.0;
}
static double disk_sigma(const vec &r) { return disk_eps(r) > 1.0 ? 0.5 : 0.0; }

static void case_aniso_bloch2d(Writer &w, int steps) {
  grid_volume gv = voltwo(1.0, 1.0, 10.0);
  structure s(gv, disk_eps, boundary_region(), identity(), 0, 0.5, true);
  s.add_susceptibility(disk_sigma, E_stuff, lorentzian_susceptibility(0.9, 0.2));
  fields f(&s);
  f.use_bloch(vec(0.3, 0.1));
  f.add_point_source(Hz, 0.5, 2.0, 0.0, 3.0, vec(0.3, 0.65), complex<double>(0.0, -1.0));
  f.add_point_source(Ey, 0.6, 2.0, 0.0, 3.0, vec(0.7, 0.2), complex<double>(0.8, 0.3));
  for (int i = 0; i < steps; i++)
    f.step();
  w.scalar("t", f.time());
  const component cs[3] = {Ex, Ey, Hz};
  const char *names[3] = {"Ex", "Ey", "Hz"};
  for (int i = 0; i < 3; i++) {
    w.rec(names[i], global_field(f, gv, cs[i]));
    w.rec(std::string(names[i]) + "_im", global_field_im(f, gv, cs[i]));
  }
  w.rec("chi_ExY", global_chi1inv(s, gv, Ex, Y));
}

// 1-D: a slab whose faces fall between grid points; averaging of the
// field parallel to the faces (harmonic mean of 1/eps)
static double slab_eps1d(const vec &r) { return r.z() > -1.03 && r.z() < 0.77 ? 4.0 : 1.0; }

static void case_aniso1d(Writer &w, int steps) {
  grid_volume gv = volone(6.0, 20.0);
  gv.center_origin();
  structure s(gv, slab_eps1d, pml(1.0), identity(), 0, 0.5, true);
  fields f(&s);
  f.use_real_fields();
  gaussian_src_time src(0.8, 0.5);
  f.add_point_source(Ex, src, vec(-1.7));
  for (int i = 0; i < steps; i++)
    f.step();
  w.scalar("t", f.time());
  w.rec("Ex", global_field(f, gv, Ex));
  w.rec("Hy", global_field(f, gv, Hy));
  w.rec("chi_ExX", global_chi1inv(s, gv, Ex, X));
}

/* Scripts with the Python front end's default eps_averaging=True.  The
   package averages its geometry with the reference's default
   material_function method (not libctl's analytic overlaps, which the
   reference's Python layer uses), so these restate the scripts as a C++
   structure built with use_anisotropic_averaging = true over a material
   function of the same objects: blocks, spheres and cylinders with any axis,
   the last containing object winning. */
struct PyAvgObj {
  int kind; // 0 block, 1 sphere, 2 cylinder
  double center[3], size[3], radius, height, axis[3];
  double eps, cond, sig;
};
class PyGeomAvg : public material_function {
public:
  int dim = 2;
  std::vector<PyAvgObj> objs;
  double eps_default = 1.0;
  static bool contains(const PyAvgObj &o, const double r[3]) {
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
  const PyAvgObj *at(const vec &r) const {
    const double p[3] = {dim == 1 ? 0.0 : r.x(), dim == 1 ? 0.0 : r.y(), dim == 2 ? 0.0 : r.z()};
    for (size_t q = objs.size(); q-- > 0;)
      if (contains(objs[q], p)) return &objs[q];
    return nullptr;
  }
  virtual double chi1p1(field_type ft, const vec &r) {
    if (ft == H_stuff) return 1.0;
    const PyAvgObj *o = at(r);
    return o ? o->eps : eps_default;
  }
  virtual bool has_conductivity(component c) {
    if (!is_D(c)) return false;
    for (const PyAvgObj &o : objs)
      if (o.cond != 0) return true;
    return false;
  }
  virtual double conductivity(component c, const vec &r) {
    const PyAvgObj *o = at(r);
    return is_D(c) && o ? o->cond : 0.0;
  }
};
class PyAvgSigma : public material_function {
public:
  const PyGeomAvg *g;
  explicit PyAvgSigma(const PyGeomAvg *geo) : g(geo) {}
  virtual void sigma_row(component c, double row[3], const vec &r) {
    row[0] = row[1] = row[2] = 0.0;
    const PyAvgObj *o = g->at(r);
    row[component_direction(c) % 3] = o ? o->sig : 0.0;
  }
};

/* Script:
     geometry = [mp.Block(mp.Vector3(mp.inf, 1, mp.inf), center=mp.Vector3(y=0.17),
                          material=mp.Medium(epsilon=12)),
                 mp.Cylinder(0.8, center=mp.Vector3(3, 1.5), material=mp.Medium(index=2)),
                 mp.Sphere(0.6, center=mp.Vector3(-2, -1.7),
                           material=mp.Medium(epsilon=6, D_conductivity=0.05))]
     sim = mp.Simulation(cell_size=mp.Vector3(16, 8), resolution=10, geometry=geometry,
                         boundary_layers=[mp.PML(1.0)],
                         sources=[mp.Source(mp.GaussianSource(0.15, fwidth=0.1), component=mp.Ey,
                                            center=mp.Vector3(-6), size=mp.Vector3(y=1))])
     tran = sim.add_flux([0.1, 0.15, 0.2], mp.FluxRegion(center=mp.Vector3(6), size=mp.Vector3(y=2)))
     sim.run(until_after_sources=20) */
static void case_py_aniso_te2d(Writer &w) {
  const double inf = 1.0e20;
  grid_volume gv = vol2d(16, 8, 10);
  gv.center_origin();
  PyGeomAvg g;
  g.dim = 2;
  g.objs = {{0, {0, 0.17, 0}, {inf, 1, inf}, 0, 0, {0, 0, 0}, 12, 0, 0},
            {2, {3, 1.5, 0}, {0, 0, 0}, 0.8, inf, {0, 0, 1}, 4, 0, 0},
            {1, {-2, -1.7, 0}, {0, 0, 0}, 0.6, 0, {0, 0, 0}, 6, 0.05, 0}};
  structure s(gv, g, pml(1.0), identity(), 0, 0.5, true, 1e-4, 100000);
  fields f(&s);
  f.use_real_fields();
  double width = std::max(0.0, 1 / 0.1);
  gaussian_src_time src(0.15, width, 0.0, 0.0 + 2 * width * 5.0);
  src.is_integrated = false;
  f.add_volume_source(Ey, src, volume(vec(-6, -0.5), vec(-6, 0.5)), complex<double>(1.0, 0.0));
  std::vector<double> fr = {0.1, 0.15, 0.2};
  volume_list r(volume(vec(6, -1), vec(6, 1)), Sx, 1.0);
  dft_flux tran = f.add_dft_flux(&r, fr.data(), fr.size(), true, true, 0);
  py_run_until_after_sources(f, 20);
  sync_dfts(f);
  double *F = tran.flux();
  w.rec("flux", std::vector<double>(F, F + fr.size()));
  delete[] F;
  w.scalar("t", f.time());
  w.rec("Ex", global_field(f, gv, Ex));
  w.rec("Ey", global_field(f, gv, Ey));
  w.rec("Hz", global_field(f, gv, Hz));
  w.rec("chi_ExY", global_chi1inv(s, gv, Ex, Y));
}

/* Script:
     mat = mp.Medium(epsilon=2.5, E_susceptibilities=[
         mp.LorentzianSusceptibility(frequency=1.1, gamma=0.1, sigma=0.5)])
     geometry = [mp.Block(mp.Vector3(1.1, 0.9, 0.73), center=mp.Vector3(0.05, -0.1, 0.02), material=mat),
                 mp.Cylinder(0.35, height=1.0, axis=mp.Vector3(0.6, 0, 0.8),
                             center=mp.Vector3(0.2, 0.3, -0.1), material=mp.Medium(epsilon=5))]
     sim = mp.Simulation(cell_size=mp.Vector3(2, 2, 2), resolution=10, geometry=geometry,
                         boundary_layers=[mp.PML(0.5)],
                         sources=[mp.Source(mp.GaussianSource(0.8, fwidth=0.5, is_integrated=True),
                                            component=mp.Ex, center=mp.Vector3(-0.4, 0.1))])
     flux = sim.add_flux(0.8, 0.4, 3, mp.FluxRegion(center=mp.Vector3(z=0.45), size=mp.Vector3(1, 1)))
     sim.run(until=6) */
static void case_py_aniso3d(Writer &w) {
  grid_volume gv = vol3d(2, 2, 2, 10);
  gv.center_origin();
  PyGeomAvg g;
  g.dim = 3;
  g.objs = {{0, {0.05, -0.1, 0.02}, {1.1, 0.9, 0.73}, 0, 0, {0, 0, 0}, 2.5, 0, 0.5},
            {2, {0.2, 0.3, -0.1}, {0, 0, 0}, 0.35, 1.0, {0.6, 0, 0.8}, 5, 0, 0}};
  structure s(gv, g, pml(0.5), identity(), 0, 0.5, true, 1e-4, 100000);
  PyAvgSigma sg(&g);
  s.add_susceptibility(sg, E_stuff, lorentzian_susceptibility(1.1, 0.1));
  fields f(&s);
  f.use_real_fields();
  double width = std::max(0.0, 1 / 0.5);
  gaussian_src_time src(0.8, width, 0.0, 0.0 + 2 * width * 5.0);
  src.is_integrated = true;
  f.add_volume_source(Ex, src, volume(vec(-0.4, 0.1, 0), vec(-0.4, 0.1, 0)), complex<double>(1.0, 0.0));
  std::vector<double> fr = np_linspace(0.8 - 0.5 * 0.4, 0.8 + 0.5 * 0.4, 3);
  volume_list r(volume(vec(-0.5, -0.5, 0.45), vec(0.5, 0.5, 0.45)), Sz, 1.0);
  dft_flux flux = f.add_dft_flux(&r, fr.data(), fr.size(), true, true, 0);
  py_run_until(f, 6);
  double *F = flux.flux();
  w.rec("flux", std::vector<double>(F, F + fr.size()));
  delete[] F;
  w.scalar("t", f.time());
  w.rec("Ex", global_field(f, gv, Ex));
  w.rec("Ez", global_field(f, gv, Ez));
  w.rec("Hy", global_field(f, gv, Hy));
  w.rec("chi_ExZ", global_chi1inv(s, gv, Ex, Z));
  w.rec("chi_EzY", global_chi1inv(s, gv, Ez, Y));
}

/* Near-to-far transform (src/near2far.cpp), after the reference's
   tests/near2far.cpp check_2d_3d: eps = 2 everywhere, two point sources at
   the origin (c0, and c1 with amplitude 0.7654321), a closed box of near2far
   surfaces at +-xmax/4, scale_dfts(sqrt(2 pi) / dt); here with Gaussian
   pulses run until they have left the cell instead of solve_cw, and no
   mirror symmetry.  Records: far fields at 20 points beyond the cell (the
   reference test's points), a far-field array over a line (2-D) or plane
   (3-D) and its flux. */
static double two_eps(const vec &) { return 2.0; }

static void write_n2f(Writer &w, dft_near2far &n2f, const std::vector<vec> &pts, const volume &arr, direction df,
                      double res) {
  const size_t nf = n2f.freq.size();
  std::vector<double> sums;
  for (dft_chunk *ch = n2f.F; ch; ch = ch->next_in_dft)
    for (size_t i = 0; i < ch->N * nf; i++) {
      sums.push_back(ch->dft[i].real());
      sums.push_back(ch->dft[i].imag());
    }
  w.rec("n2f_dft", sums);
  w.scalar("n2f_eps", n2f.eps);
  w.scalar("n2f_mu", n2f.mu);
  std::vector<double> ff;
  for (const vec &x : pts) {
    complex<double> *EH = n2f.farfield(x);
    for (size_t i = 0; i < 6 * nf; i++) {
      ff.push_back(EH[i].real());
      ff.push_back(EH[i].imag());
    }
    delete[] EH;
  }
  w.rec("ff", ff);
  std::vector<double> xs;
  for (const vec &x : pts)
    for (int d = 0; d < 3; d++)
      xs.push_back(d < 2 || x.dim == D3 ? x.in_direction(direction(d)) : 0.0);
  w.rec("ff_points", xs);
  int rank = 0;
  size_t dims[3] = {1, 1, 1}, N = 1;
  double *EH = n2f.get_farfields_array(arr, rank, dims, N, res);
  w.rec("ffarr", std::vector<double>(EH, EH + 12 * N * nf));
  w.rec("ffarr_dims", std::vector<double>{double(rank), double(dims[0]), double(dims[1]), double(dims[2])});
  delete[] EH;
  double *F = n2f.flux(df, arr, res);
  w.rec("ffflux", std::vector<double>(F, F + nf));
  delete[] F;
}

static void case_n2f(Writer &w, ndim dim, component c0, component c1, int steps) {
  const double dpml = 1, xmax = dim == D2 ? 4 : 3, a = dim == D2 ? 20 : 10;
  grid_volume gv = dim == D2 ? vol2d(xmax + 2 * dpml, xmax + 2 * dpml, a)
                             : vol3d(xmax + 2 * dpml, xmax + 2 * dpml, xmax + 2 * dpml, a);
  gv.center_origin();
  structure s(gv, two_eps, pml(dpml), identity(), 0, 0.5, false);
  fields f(&s);
  f.use_real_fields();
  const double w0 = dim == D2 ? 0.3 : 0.5;
  // same pulse for both; a current (not integrated) source where it is
  // magnetic, the only kind this engine takes on H
  gaussian_src_time src(w0, dim == D2 ? 0.2 : 0.3), srcm(w0, dim == D2 ? 0.2 : 0.3);
  srcm.is_integrated = false;
  f.add_point_source(c0, is_magnetic(c0) ? srcm : src, zero_vec(dim));
  f.add_point_source(c1, is_magnetic(c1) ? srcm : src, zero_vec(dim), 0.7654321);
  const double L = xmax / 4;
  volume_list *vl;
  if (dim == D2)
    vl = new volume_list(
        volume(vec(-L, +L), vec(+L, +L)), Sy, 1.0,
        new volume_list(volume(vec(+L, +L), vec(+L, -L)), Sx, 1.0,
                        new volume_list(volume(vec(-L, -L), vec(+L, -L)), Sy, -1.0,
                                        new volume_list(volume(vec(-L, -L), vec(-L, +L)), Sx, -1.0))));
  else
    vl = new volume_list(
        volume(vec(+L, -L, -L), vec(+L, +L, +L)), Sx, +1.,
        new volume_list(
            volume(vec(-L, -L, -L), vec(-L, +L, +L)), Sx, -1.,
            new volume_list(
                volume(vec(-L, +L, -L), vec(+L, +L, +L)), Sy, +1.,
                new volume_list(volume(vec(-L, -L, -L), vec(+L, -L, +L)), Sy, -1.,
                                new volume_list(volume(vec(-L, -L, +L), vec(+L, +L, +L)), Sz, +1.,
                                                new volume_list(volume(vec(-L, -L, -L), vec(+L, +L, -L)),
                                                                Sz, -1.))))));
  std::vector<double> fr = {w0 - 0.05, w0, w0 + 0.05};
  dft_near2far n2f = f.add_dft_near2far(vl, fr.data(), fr.size(), 0, 1);
  delete vl;
  for (int i = 0; i < steps; i++)
    f.step();
  w.scalar("t", f.time());
  n2f.scale_dfts(std::sqrt(2 * pi) / f.dt);
  sync_dfts(f);
  const int N = 20;
  const double dx = 0.75 * (xmax / 4) / N;
  std::vector<vec> pts;
  for (int i = 0; i < N; ++i) {
    const double sx = xmax + dx * i;
    pts.push_back(dim == D2 ? vec(sx, 0.5 * sx) : vec(sx, 0.5 * sx, 0.3 * sx));
  }
  if (dim == D2) write_n2f(w, n2f, pts, volume(vec(6, -3), vec(6, 3)), X, 4.0);
  else write_n2f(w, n2f, pts, volume(vec(4, -2, -2), vec(4, 2, 2)), X, 3.0);
}

// periodic in x (Bloch), PML in y: a near2far line spanning the cell width,
// summed over 2 * 3 + 1 lattice images with the Bloch phase
static double eps15(const vec &) { return 1.5; }

static void case_n2f_periodic2d(Writer &w, int steps) {
  grid_volume gv = vol2d(2.0, 6.0, 20.0);
  gv.center_origin();
  structure s(gv, eps15, pml(1.0, Y), identity(), 0, 0.5, false);
  fields f(&s);
  f.use_bloch(X, 0.15);
  gaussian_src_time src(0.6, 0.4), srcm(0.6, 0.4);
  srcm.is_integrated = false;
  f.add_point_source(Ez, src, vec(0.2, -1.0));
  f.add_point_source(Hx, srcm, vec(-0.3, -0.8), complex<double>(0.3, 0.2));
  volume_list vl(volume(vec(-1.0, 1.0), vec(1.0, 1.0)), Sy, 1.0);
  std::vector<double> fr = {0.5, 0.6, 0.7};
  dft_near2far n2f = f.add_dft_near2far(&vl, fr.data(), fr.size(), 0, 3);
  for (int i = 0; i < steps; i++)
    f.step();
  w.scalar("t", f.time());
  sync_dfts(f);
  std::vector<vec> pts;
  for (int i = 0; i < 12; ++i)
    pts.push_back(vec(-1.5 + 0.27 * i, 3.0 + 0.4 * i));
  write_n2f(w, n2f, pts, volume(vec(-2, 5), vec(2, 5)), Y, 5.0);
  w.scalar("n2f_periodic_n", n2f.periodic_n[1]);
  w.scalar("n2f_periodic_k", n2f.periodic_k[1]);
}

/* Script (the reference's python/tests/test_antenna_radiation.py
   test_poynting_theorem at resolution 20, no mirror symmetry, a fixed run
   time instead of stop_when_fields_decayed):
     sim = mp.Simulation(cell_size=mp.Vector3(6, 6), resolution=20, boundary_layers=[mp.PML(1)],
                         sources=[mp.Source(mp.GaussianSource(1.0, fwidth=0.4), center=mp.Vector3(),
                                            component=mp.Ez)], eps_averaging=False)
     n2f = sim.add_near2far(1.0, 0, 1, <the four sides of the 4 x 4 box, weights +1, -1, +1, -1>)
     box = sim.add_flux(1.0, 0, 1, <the same four regions>)
     sim.run(until_after_sources=40)
     near = mp.get_fluxes(box)[0]
     ff = [sim.get_farfield(n2f, mp.Vector3(1000 * sin(a), 1000 * cos(a))) for 12 angles a in [0, pi/2)]
     square = [n2f.flux(d, mp.Volume(center=..., size=...), 20) for the four sides of a 20 x 20 square]
     arr = sim.get_farfields(n2f, resolution=2, center=mp.Vector3(0, 6), size=mp.Vector3(10, 0)) */
static void case_py_n2f(Writer &w) {
  grid_volume gv = vol2d(6, 6, 20);
  gv.center_origin();
  structure s(gv, one_eps, pml(1.0), identity(), 0, 0.5, false);
  fields f(&s);
  f.use_real_fields();
  const double fcen = 1.0, df = 0.4, sxy = 4;
  double width = std::max(0.0, 1 / df);
  gaussian_src_time src(fcen, width, 0.0, 0.0 + 2 * width * 5.0);
  src.is_integrated = false;
  f.add_volume_source(Ez, src, volume(vec(0, 0), vec(0, 0)), complex<double>(1.0, 0.0));
  // regions in script order; the Python layer prepends each to the list
  struct Reg {
    vec c, sz;
    double wgt;
  } regs[4] = {{vec(0, 0.5 * sxy), vec(sxy, 0), 1.0},
               {vec(0, -0.5 * sxy), vec(sxy, 0), -1.0},
               {vec(0.5 * sxy, 0), vec(0, sxy), 1.0},
               {vec(-0.5 * sxy, 0), vec(0, sxy), -1.0}};
  auto vlist = [&]() {
    volume_list *vl = nullptr;
    for (const Reg &r : regs) {
      volume v(r.c - r.sz * 0.5, r.c + r.sz * 0.5);
      vl = new volume_list(v, r.sz.x() == 0 ? Sx : Sy, r.wgt, vl);
    }
    return vl;
  };
  std::vector<double> fr = {fcen};
  volume_list *l1 = vlist();
  dft_near2far n2f = f.add_dft_near2far(l1, fr.data(), fr.size(), 0, 1);
  delete l1;
  volume_list *l2 = vlist();
  dft_flux box = f.add_dft_flux(l2, fr.data(), fr.size(), true, true, 0);
  delete l2;
  py_run_until_after_sources(f, 40);
  sync_dfts(f);
  double *F = box.flux();
  w.scalar("near_flux", F[0]);
  delete[] F;
  w.scalar("t", f.time());
  std::vector<double> ff;
  for (int i = 0; i < 12; i++) {
    const double ang = 0.5 * pi / 12 * i, r = 1000 / fcen;
    complex<double> *EH = n2f.farfield(vec(r * std::sin(ang), r * std::cos(ang)));
    for (int j = 0; j < 6; j++) {
      ff.push_back(EH[j].real());
      ff.push_back(EH[j].imag());
    }
    delete[] EH;
  }
  w.rec("ff", ff);
  const double rr = 20 / fcen;
  const direction dirs[4] = {Y, Y, X, X};
  const vec cen[4] = {vec(0, 0.5 * rr), vec(0, -0.5 * rr), vec(0.5 * rr, 0), vec(-0.5 * rr, 0)};
  const vec siz[4] = {vec(rr, 0), vec(rr, 0), vec(0, rr), vec(0, rr)};
  std::vector<double> sq;
  for (int k = 0; k < 4; k++) {
    double *Fk = n2f.flux(dirs[k], volume(cen[k] - siz[k] * 0.5, cen[k] + siz[k] * 0.5), 20);
    sq.push_back(Fk[0]);
    delete[] Fk;
  }
  w.rec("square_flux", sq);
  int rank = 0;
  size_t dims[3] = {1, 1, 1}, N = 1;
  double *EH = n2f.get_farfields_array(volume(vec(-5, 6), vec(5, 6)), rank, dims, N, 2.0);
  w.rec("ffarr", std::vector<double>(EH, EH + 12 * N));
  delete[] EH;
}

// run(until_after_sources=stop_when_fields_decayed(dt, c, pt, decay_by))
// (python/simulation.py:5275-5336 with _run_sources_until :2866-2885): the
// condition samples |c(pt)|^2 on every step and stops once the largest value
// of the last dt window is below decay_by times the largest before it, and
// the sources are off
static void py_run_until_after_sources_decayed(fields &f, double dt, component c, const vec &pt, double decay_by) {
  double max_abs = 0, cur_max = 0, t0 = 0;
  const double ts = f.last_source_time();
  auto stop = [&]() {
    const double a = std::abs(f.get_field(c, pt));
    cur_max = std::max(cur_max, a * a);
    if (f.round_time() <= dt + t0) return false;
    const double old = cur_max;
    cur_max = 0;
    t0 = f.round_time();
    max_abs = std::max(max_abs, old);
    return old <= max_abs * decay_by;
  };
  while (!(stop() && f.round_time() >= ts))
    f.step();
}

/* Script (the reference's python/tests/test_force.py test_force):
     sim = mp.Simulation(resolution=20, cell_size=mp.Vector3(10, 10), boundary_layers=[mp.PML(1.0)],
                         sources=[mp.Source(mp.GaussianSource(1.0, fwidth=1.0), center=mp.Vector3(),
                                            component=mp.Ez)])
     fr = mp.ForceRegion(center=mp.Vector3(0, 1.27), direction=mp.Y, size=mp.Vector3(4.38, 0))
     force = sim.add_force(1.0, 0, 1, fr, decimation_factor=1)
     force_decimated = sim.add_force(1.0, 0, 1, fr, decimation_factor=10)
     sim.run(until_after_sources=mp.stop_when_fields_decayed(50, mp.Ez, mp.Vector3(), 1e-6))
   (its golden master: get_forces(force)[0] = -0.11039089113393187) */
static void case_py_force(Writer &w) {
  grid_volume gv = vol2d(10, 10, 20);
  gv.center_origin();
  structure s(gv, one_eps, pml(1.0), identity(), 0, 0.5, true);
  fields f(&s);
  f.use_real_fields();
  double width = std::max(0.0, 1 / 1.0);
  gaussian_src_time src(1.0, width, 0.0, 0.0 + 2 * width * 5.0);
  src.is_integrated = false;
  f.add_volume_source(Ez, src, volume(vec(0, 0), vec(0, 0)), complex<double>(1.0, 0.0));
  std::vector<double> fr = {1.0};
  volume_list r(volume(vec(-2.19, 1.27), vec(2.19, 1.27)), Sy, 1.0);
  dft_force force = f.add_dft_force(&r, fr.data(), fr.size(), 1);
  dft_force force_dec = f.add_dft_force(&r, fr.data(), fr.size(), 10);
  // and the test's fr_box: force along x on the four sides of a 2 x 2 box
  // (diagonal stress terms on the x sides, off-diagonal on the y sides)
  volume_list *box = nullptr;
  const double bc[4][2] = {{1.0, 0}, {-1.0, 0}, {0, 1.0}, {0, -1.0}}, bw[4] = {1.0, -1.0, 1.0, -1.0};
  for (int q = 0; q < 4; q++) {
    const double hx = q < 2 ? 0.0 : 1.0, hy = q < 2 ? 1.0 : 0.0;
    box = new volume_list(volume(vec(bc[q][0] - hx, bc[q][1] - hy), vec(bc[q][0] + hx, bc[q][1] + hy)), Sx, bw[q],
                          box);
  }
  dft_force force_box = f.add_dft_force(box, fr.data(), fr.size(), 1);
  delete box;
  py_run_until_after_sources_decayed(f, 50, Ez, vec(0, 0), 1e-6);
  sync_dfts(f);
  double *F = force.force();
  w.scalar("force", F[0]);
  delete[] F;
  F = force_dec.force();
  w.scalar("force_dec", F[0]);
  delete[] F;
  F = force_box.force();
  w.scalar("force_box", F[0]);
  delete[] F;
  w.scalar("t", f.time());
  w.rec("Ez", global_field(f, gv, Ez));
}

/* Script (the reference's python/tests/test_dft_energy.py with a line source
   across the guide instead of the eigenmode source, resolution 10, 50 time
   units after the sources):
     sim = mp.Simulation(resolution=10, cell_size=mp.Vector3(10, 5), eps_averaging=False,
                         geometry=[mp.Block(size=mp.Vector3(mp.inf, 1, mp.inf), material=mp.Medium(epsilon=12))],
                         boundary_layers=[mp.PML(1)],
                         sources=[mp.Source(mp.GaussianSource(0.15, fwidth=0.03), component=mp.Ez,
                                            center=mp.Vector3(-3), size=mp.Vector3(y=5))])
     flux = sim.add_flux(0.15, 0, 1, mp.FluxRegion(center=mp.Vector3(3), size=mp.Vector3(y=5)), decimation_factor=1)
     energy = sim.add_energy(0.15, 0, 1, mp.EnergyRegion(center=mp.Vector3(3), size=mp.Vector3(y=5)),
                             decimation_factor=1)
     energy_decimated = (the same with decimation_factor=10)
     sim.run(until_after_sources=50) */
static void case_py_energy(Writer &w) {
  const double inf = 1.0e20;
  grid_volume gv = vol2d(10, 5, 10);
  gv.center_origin();
  PyGeom g;
  g.dim = 2;
  g.meds = {{{1, 1, 1}, 0, {0, 0}}, {{12, 12, 12}, 0, {0, 0}}};
  g.objs = {{0, {0, 0, 0}, {inf, 1, inf}, 0, 1}};
  structure s(gv, g, pml(1.0), identity(), 0, 0.5, false);
  fields f(&s);
  f.use_real_fields();
  double width = std::max(0.0, 1 / 0.03);
  gaussian_src_time src(0.15, width, 0.0, 0.0 + 2 * width * 5.0);
  src.is_integrated = false;
  f.add_volume_source(Ez, src, volume(vec(-3, -2.5), vec(-3, 2.5)), complex<double>(1.0, 0.0));
  std::vector<double> fr = {0.15};
  volume_list r(volume(vec(3, -2.5), vec(3, 2.5)), Sx, 1.0);
  dft_flux flux = f.add_dft_flux(&r, fr.data(), fr.size(), true, true, 1);
  dft_energy energy = f.add_dft_energy(&r, fr.data(), fr.size(), 1);
  dft_energy energy_dec = f.add_dft_energy(&r, fr.data(), fr.size(), 10);
  py_run_until_after_sources(f, 50);
  sync_dfts(f);
  double *F = flux.flux();
  w.scalar("flux", F[0]);
  delete[] F;
  dft_energy *es[2] = {&energy, &energy_dec};
  const char *names[2] = {"", "_dec"};
  for (int q = 0; q < 2; q++) {
    F = es[q]->electric();
    w.scalar(std::string("electric") + names[q], F[0]);
    delete[] F;
    F = es[q]->magnetic();
    w.scalar(std::string("magnetic") + names[q], F[0]);
    delete[] F;
    F = es[q]->total();
    w.scalar(std::string("total") + names[q], F[0]);
    delete[] F;
  }
  w.scalar("t", f.time());
}

/* Script (dft_ldos as in the reference's python/tests/test_ldos.py, here in
   2-D Cartesian with a dielectric block beside an off-grid dipole):
     sim = mp.Simulation(cell_size=mp.Vector3(6, 6), resolution=20, boundary_layers=[mp.PML(1)],
                         eps_averaging=False,
                         geometry=[mp.Block(mp.Vector3(1, 1, mp.inf), center=mp.Vector3(0.8),
                                            material=mp.Medium(epsilon=4))],
                         sources=[mp.Source(mp.GaussianSource(1.0, fwidth=0.2), component=mp.Ez,
                                            center=mp.Vector3(0.1, 0.05))])
     sim.run(mp.dft_ldos(1.0, 0.2, 5), until_after_sources=20)
     sim.ldos_data, sim.ldos_Fdata, sim.ldos_Jdata */
/* Script (the weights u: mt19937_64(77) uniform [0, 1), 15 x 11, written to
   the fixture as "weights"):
     mg = mp.MaterialGrid(mp.Vector3(15, 11), mp.Medium(epsilon=1.5), mp.Medium(epsilon=9),
                          weights=u, beta=6, eta=0.45)
     geometry = [mp.Cylinder(0.6, center=mp.Vector3(-2, 1.5), material=mp.Medium(epsilon=4)),
                 mp.Block(center=mp.Vector3(0.3, -0.2), size=mp.Vector3(3.1, 2.3), material=mg)]
     sim = mp.Simulation(cell_size=mp.Vector3(10, 8), resolution=10, geometry=geometry,
                         boundary_layers=[mp.PML(1.0)], eps_averaging=False,
                         sources=[mp.Source(mp.GaussianSource(0.2, fwidth=0.2), component=mp.Ez,
                                            center=mp.Vector3(-3, 0))])
     flux = sim.add_flux(0.2, 0.2, 5, mp.FluxRegion(center=mp.Vector3(3), size=mp.Vector3(0, 4)))
     sim.run(until=60)
   The grid material as the reference's geometry evaluates it without
   smoothing: the weights linearly interpolated at the point's block
   coordinates (linear_interpolate with mirror faces, src/fields.cpp:759-806),
   projected (tanh_projection, src/meepgeom.cpp:497-502), eps1 + u (eps2 -
   eps1) (epsilon_material_grid, :569-581). */
class PyMatGridGeom : public material_function {
public:
  double bc[3] = {0.3, -0.2, 0.0}, bs[3] = {3.1, 2.3, 0.0};
  int n[3] = {15, 11, 1};
  std::vector<double> u;
  double beta = 6, eta = 0.45, e1 = 1.5, e2 = 9.0;
  static int mirror(int i, int m) { return i >= m ? 2 * m - 1 - i : (i < 0 ? -1 - i : i); }
  double interp(const double r0[3]) const {
    int i1[3], i2[3];
    double w[3];
    for (int d = 0; d < 3; d++) {
      double r = r0[d] < 0.0 ? -r0[d] : (r0[d] > 1.0 ? 1.0 - r0[d] : r0[d]);
      i1[d] = mirror(int(r * n[d]), n[d]);
      double dd = r * n[d] - i1[d] - 0.5;
      i2[d] = mirror(dd >= 0.0 ? i1[d] + 1 : i1[d] - 1, n[d]);
      w[d] = std::fabs(dd);
    }
    auto U = [&](int x, int y, int z) { return u[(x * n[1] + y) * n[2] + z]; };
    return (((U(i1[0], i1[1], i1[2]) * (1.0 - w[0]) + U(i2[0], i1[1], i1[2]) * w[0]) * (1.0 - w[1]) +
             (U(i1[0], i2[1], i1[2]) * (1.0 - w[0]) + U(i2[0], i2[1], i1[2]) * w[0]) * w[1]) *
                (1.0 - w[2]) +
            ((U(i1[0], i1[1], i2[2]) * (1.0 - w[0]) + U(i2[0], i1[1], i2[2]) * w[0]) * (1.0 - w[1]) +
             (U(i1[0], i2[1], i2[2]) * (1.0 - w[0]) + U(i2[0], i2[1], i2[2]) * w[0]) * w[1]) *
                w[2]);
  }
  double eps_at(const vec &v) const {
    const double p[3] = {v.x(), v.y(), 0.0};
    bool in = true;
    for (int d = 0; d < 3; d++)
      in = in && std::fabs(p[d] - bc[d]) <= 0.5 * bs[d];
    if (in) {
      double r[3];
      for (int d = 0; d < 3; d++)
        r[d] = bs[d] == 0 ? 0.0 : 0.5 + (p[d] - bc[d]) / bs[d];
      double x = interp(r);
      if (beta != 0) {
        const double t = std::tanh(beta * eta);
        x = x == eta ? 0.5 : (t + std::tanh(beta * (x - eta))) / (t + std::tanh(beta * (1 - eta)));
      }
      return e1 + x * (e2 - e1);
    }
    const double dx = p[0] + 2, dy = p[1] - 1.5;
    return dx * dx + dy * dy <= 0.6 * 0.6 ? 4.0 : 1.0;
  }
  virtual double chi1p1(field_type ft, const vec &r) { return ft == H_stuff ? 1.0 : eps_at(r); }
  virtual void eff_chi1inv_row(component c, double row[3], const volume &v, double, int) {
    row[0] = row[1] = row[2] = 0.0;
    row[component_direction(c) % 3] = type(c) == H_stuff ? 1.0 : 1.0 / eps_at(v.center());
  }
};

static void case_py_matgrid(Writer &w) {
  grid_volume gv = vol2d(10, 8, 10);
  gv.center_origin();
  PyMatGridGeom g;
  std::mt19937_64 rng(77);
  std::uniform_real_distribution<double> uni(0.0, 1.0);
  g.u.resize(15 * 11);
  for (double &x : g.u)
    x = uni(rng);
  w.rec("weights", g.u);
  structure s(gv, g, pml(1.0), identity(), 0, 0.5, false);
  fields f(&s);
  f.use_real_fields();
  double width = std::max(0.0, 1 / 0.2);
  gaussian_src_time src(0.2, width, 0.0, 0.0 + 2 * width * 5.0);
  src.is_integrated = false;
  f.add_volume_source(Ez, src, volume(vec(-3, 0), vec(-3, 0)), complex<double>(1.0, 0.0));
  std::vector<double> fr = np_linspace(0.2 - 0.5 * 0.2, 0.2 + 0.5 * 0.2, 5);
  volume_list r1(volume(vec(3, -2), vec(3, 2)), Sx, 1.0);
  dft_flux fl = f.add_dft_flux(&r1, fr.data(), fr.size(), true, true, 0);
  py_run_until(f, 60);
  sync_dfts(f);
  double *F = fl.flux();
  w.rec("flux", std::vector<double>(F, F + fr.size()));
  delete[] F;
  w.scalar("t", f.time());
  w.rec("Ez", global_field(f, gv, Ez));
}

static void case_py_ldos(Writer &w) {
  const double inf = 1.0e20;
  grid_volume gv = vol2d(6, 6, 20);
  gv.center_origin();
  PyGeom g;
  g.dim = 2;
  g.meds = {{{1, 1, 1}, 0, {0, 0}}, {{4, 4, 4}, 0, {0, 0}}};
  g.objs = {{0, {0.8, 0, 0}, {1, 1, inf}, 0, 1}};
  structure s(gv, g, pml(1.0), identity(), 0, 0.5, false);
  fields f(&s);
  f.use_real_fields();
  double width = std::max(0.0, 1 / 0.2);
  gaussian_src_time src(1.0, width, 0.0, 0.0 + 2 * width * 5.0);
  src.is_integrated = false;
  f.add_volume_source(Ez, src, volume(vec(0.1, 0.05), vec(0.1, 0.05)), complex<double>(1.0, 0.0));
  std::vector<double> fr = np_linspace(1.0 - 0.5 * 0.2, 1.0 + 0.5 * 0.2, 5);
  dft_ldos ldos(fr.data(), fr.size());
  // run(step function, until_after_sources=20): the step function before
  // every step and once after the last
  const double ts = f.last_source_time();
  const double until = (ts - f.round_time()) + 20, t0 = f.round_time();
  while (!(f.round_time() >= t0 + until)) {
    ldos.update(f);
    f.step();
  }
  ldos.update(f);
  double *L = ldos.ldos();
  w.rec("ldos", std::vector<double>(L, L + fr.size()));
  delete[] L;
  complex<double> *F = ldos.F(), *J = ldos.J();
  std::vector<double> vf, vj;
  for (size_t i = 0; i < fr.size(); i++) {
    vf.push_back(F[i].real());
    vf.push_back(F[i].imag());
    vj.push_back(J[i].real());
    vj.push_back(J[i].imag());
  }
  delete[] F;
  delete[] J;
  w.rec("F", vf);
  w.rec("J", vj);
  w.scalar("t", f.time());
}

#ifndef MEEP_GB300
/* ------------------------------------------------------------ adjoint_tm2d
   The reference's adjoint-solver gradient for a pixel-permittivity design
   (2-D TM), for comparison with the engine's reverse-time gradient.
   Reference core only: it calls dft_fields::fourier_sourcedata and
   fields::add_srcdata (src/dft.cpp:1491-1590, src/sources.cpp:314-338),
   which the drop-in does not carry.

   Cell 10 x 6 at resolution 10 (100 x 60 pixels), PML 1 on every side, an
   eps = 12 guide on the Ez rows |y| <= 0.4, a 20 x 20-pixel design block on
   the Ez points x, y in [-1, 0.9] with eps = eps1 + u (eps2 - eps1), u drawn
   from mt19937_64(2024); Gaussian Ez current line source (f 0.15, fwidth
   0.1, not integrated) across the guide at x = -3; J = sum |F|^2 over the
   Ez DFT (f 0.15, Yee grid) on the line x = 3, |y| <= 1.  Real fields, DFT
   decimation 1.

   The steps of the reference's Python adjoint layer, restated in C++:
     forward   FourierFields.register_monitors (python/adjoint/objective.py:
               358-368) and the design-region Dz DFT on the Yee grid
               (python/adjoint/utils.py:160-178: Dx, Dy, Dz; TM has Dz only);
               NFWD steps, so the forward time covers the adjoint profile
               that _adj_src_scale transforms over [0, T)
     dJ        autograd's convention for a real function of complex F,
               dJ/dRe F - i dJ/dIm F = 2 conj(F)
     adjoint   FourierFields.place_adjoint_source (objective.py:370-416):
               fourier_sourcedata(dJ) amplitudes times _adj_src_scale
               (objective.py:65-136; include_resolution False; one frequency:
               dV * iomega / fwd_dtft / adj_src_phase, times 2 for real
               fields), time profile GaussianSource(f, 0.1 f, cutoff 5)
               (objective.py:139-153), on fresh fields (restart_fields), the
               design-region Dz DFT, NADJ steps (sources end at t = 666.7)
     gradient  material_grids_addgradient (src/meepgeom.cpp:2835-3011) for a
               material grid whose nodes are the design block's Ez points,
               no smoothing and beta = 0, so every Ez point meets one node
               with weight 1 (add_interpolate_weights, :2710-2756): it adds
               Re[adj * fwd (chi1inv(u - du) - chi1inv(u + du)) / 2du],
               du = 1e-3 (utils.py FD_DEFAULT), chi1inv(u) = 1 / (eps1 +
               u (eps2 - eps1)) (epsilon_material_grid, :569-581)
   Central differences of J on the reference core at the four pixels with
   the largest gradient, and along a random direction, pin the restatement. */
namespace adj2d {
const int NX = 100, NY = 60;
const double RES = 10.0;
const double EPS1 = 1.5, EPS2 = 6.0, EPS_GUIDE = 12.0;
const int DI0 = 40, DJ0 = 20, DN = 20;
const double F0 = 0.15;
const int NFWD = 14000, NADJ = 16000;

class PixelEps : public material_function {
public:
  std::vector<double> eps; // Ez points (NX + 1) x (NY + 1), x-major
  double at(const vec &r) const {
    long i = lround((r.x() + 0.5 * NX / RES) * RES), j = lround((r.y() + 0.5 * NY / RES) * RES);
    i = std::min<long>(std::max<long>(i, 0), NX);
    j = std::min<long>(std::max<long>(j, 0), NY);
    return eps[i * (NY + 1) + j];
  }
  virtual double chi1p1(field_type ft, const vec &r) { return ft == H_stuff ? 1.0 : at(r); }
  virtual void eff_chi1inv_row(component c, double row[3], const volume &v, double tol, int maxeval) {
    (void)tol;
    (void)maxeval;
    row[0] = row[1] = row[2] = 0.0;
    row[component_direction(c) % 3] = type(c) == H_stuff ? 1.0 : 1.0 / at(v.center());
  }
};

static grid_volume gvol() {
  grid_volume gv = vol2d(NX / RES, NY / RES, RES);
  gv.center_origin();
  return gv;
}
static volume source_line() { return volume(vec(-3.0, -0.45), vec(-3.0, 0.45)); }
static volume obj_vol() { return volume(vec(3.0, -1.0), vec(3.0, 1.0)); }
static volume design_vol() { return volume(vec(-1.0, -1.0), vec(0.9, 0.9)); }

static void add_forward_source(fields &f) {
  double width = std::max(0.0, 1 / 0.1);
  gaussian_src_time src(F0, width, 0.0, 0.0 + 2 * width * 5.0);
  src.is_integrated = false;
  f.add_volume_source(Ez, src, source_line(), complex<double>(1.0, 0.0));
}

/* (ivec coordinates, value) of every point of a one-frequency DFT */
static std::map<std::vector<int>, complex<double> > dft_points(dft_chunk *chunks, component c,
                                                                const grid_volume &gv) {
  std::map<std::vector<int>, complex<double> > out;
  std::vector<double> flat = dump_dft_chunks(chunks, c, gv);
  const size_t rec = 2 + 2;
  for (size_t k = 0; k + rec <= flat.size(); k += rec)
    out[{int(flat[k]), int(flat[k + 1])}] = complex<double>(flat[k + 2], flat[k + 3]);
  return out;
}

/* J = sum |F|^2 of a forward run with the given permittivity */
static double forward_J(const std::vector<double> &eps) {
  grid_volume gv = gvol();
  PixelEps mat;
  mat.eps = eps;
  structure s(gv, mat, pml(1.0), identity(), 0, 0.5, false);
  fields f(&s);
  f.use_real_fields();
  add_forward_source(f);
  component cz = Ez;
  double fr = F0;
  dft_fields obj = f.add_dft_fields(&cz, 1, obj_vol(), &fr, 1, false, 1, false);
  for (int n = 0; n < NFWD; n++)
    f.step();
  double J = 0;
  for (auto &kv : dft_points(obj.chunks, Ez, gv))
    J += std::norm(kv.second);
  return J;
}
} // namespace adj2d

static void case_adjoint_tm2d(Writer &w) {
  using namespace adj2d;
  grid_volume gv = gvol();
  std::vector<double> eps((NX + 1) * (NY + 1), 1.0);
  for (int i = 0; i <= NX; i++)
    for (int j = 26; j <= 34; j++)
      eps[i * (NY + 1) + j] = EPS_GUIDE;
  std::mt19937_64 rng(2024);
  std::uniform_real_distribution<double> uni(0.0, 1.0);
  std::vector<double> u(DN * DN);
  for (int a = 0; a < DN; a++)
    for (int b = 0; b < DN; b++) {
      u[a * DN + b] = uni(rng);
      eps[(DI0 + a) * (NY + 1) + DJ0 + b] = EPS1 + u[a * DN + b] * (EPS2 - EPS1);
    }
  w.rec("eps", eps);
  w.rec("u", u);
  w.rec("eps12", {EPS1, EPS2});
  w.rec("design_lo_n", {double(DI0), double(DJ0), double(DN)});
  w.rec("steps", {double(NFWD), double(NADJ)});

  PixelEps mat;
  mat.eps = eps;
  structure s(gv, mat, pml(1.0), identity(), 0, 0.5, false);

  /* forward */
  fields f(&s);
  f.use_real_fields();
  add_forward_source(f);
  std::vector<double> srcpts; // ivec x, y, Re amp, Im amp
  for (int ic = 0; ic < f.num_chunks; ic++) {
    fields_chunk *fc = f.chunks[ic];
    if (!fc->is_mine()) continue;
    for (int ft = 0; ft < NUM_FIELD_TYPES; ft++)
      for (const meep::src_vol &sv : fc->sources[ft])
        for (size_t j = 0; j < sv.num_points(); j++) {
          ivec iv = fc->gv.iloc(sv.c, sv.index_at(j));
          srcpts.push_back(iv.x());
          srcpts.push_back(iv.y());
          srcpts.push_back(sv.amplitude_at(j).real());
          srcpts.push_back(sv.amplitude_at(j).imag());
        }
  }
  w.rec("src_points", srcpts);
  component cz = Ez, cdz = Dz;
  double fr = F0;
  dft_fields obj = f.add_dft_fields(&cz, 1, obj_vol(), &fr, 1, false, 1, false);
  dft_fields fwd_design = f.add_dft_fields(&cdz, 1, design_vol(), &fr, 1, false, 1, false);
  for (int n = 0; n < NFWD; n++)
    f.step();
  std::map<std::vector<int>, complex<double> > F = dft_points(obj.chunks, Ez, gv);
  std::vector<double> rec_F;
  double J = 0;
  int ymin = 1 << 30;
  for (auto &kv : F) {
    rec_F.insert(rec_F.end(), {double(kv.first[0]), double(kv.first[1]), kv.second.real(), kv.second.imag()});
    J += std::norm(kv.second);
    ymin = std::min(ymin, kv.first[1]);
  }
  w.rec("obj_F", rec_F);
  w.scalar("J", J);

  /* dJ in the monitor's array order (points along y) */
  std::vector<complex<double> > dJ(F.size());
  for (auto &kv : F)
    dJ[(kv.first[1] - ymin) / 2] = 2.0 * std::conj(kv.second);

  /* _adj_src_scale */
  const double T = f.time(), dt = f.dt;
  const double width_adj = std::max(0.0, 1 / (0.1 * F0));
  gaussian_src_time prof(F0, width_adj, 0.0, 0.0 + 2 * width_adj * 5);
  prof.is_integrated = false;
  const complex<double> iomega = (1.0 - std::exp(complex<double>(-0.0, -(2 * pi * F0)) * dt)) * (1.0 / dt);
  const size_t nt = size_t(std::ceil(T / dt));
  complex<double> dtft = 0;
  for (size_t k = 0; k < nt; k++) {
    const double ph = (((2 * pi) * F0) * double(k)) * dt;
    dtft += std::polar(1.0, ph) * prof.current(double(k) * dt, dt);
  }
  dtft = dtft * dt / std::sqrt(2 * pi);
  const complex<double> fwidth_scale = std::exp(complex<double>(-0.0, -2 * pi) * 5.0 / 0.1);
  const complex<double> phase = std::polar(1.0, std::arg(dtft)) * fwidth_scale;
  const complex<double> scale = 1.0 * iomega / dtft / phase * 2.0;
  w.rec("adj_scale", {T, dtft.real(), dtft.imag(), scale.real(), scale.imag()});

  /* adjoint */
  std::vector<sourcedata> sd = obj.fourier_sourcedata(obj_vol(), Ez, f, dJ.data());
  fields f2(&s);
  f2.use_real_fields();
  for (sourcedata &d : sd) {
    std::vector<complex<double> > amps(d.amp_arr.size());
    for (size_t k = 0; k < amps.size(); k++)
      amps[k] = d.amp_arr[k] * scale;
    f2.add_srcdata(d, &prof, amps.size(), amps.data(), false);
  }
  f2.require_source_components();
  dft_fields adj_design = f2.add_dft_fields(&cdz, 1, design_vol(), &fr, 1, false, 1, false);
  for (int n = 0; n < NADJ; n++)
    f2.step();

  /* material_grids_addgradient for the pixel grid */
  std::map<std::vector<int>, complex<double> > fw = dft_points(fwd_design.chunks, Dz, gv);
  std::map<std::vector<int>, complex<double> > ad = dft_points(adj_design.chunks, Dz, gv);
  const double du = 1e-3;
  std::vector<double> grad(DN * DN, 0.0), rec_design;
  for (auto &kv : ad) {
    const int i = (kv.first[0] + NX) / 2, j = (kv.first[1] + NY) / 2;
    const int a = i - DI0, b = j - DJ0;
    const complex<double> fv = fw.at(kv.first);
    rec_design.insert(rec_design.end(), {double(kv.first[0]), double(kv.first[1]), fv.real(), fv.imag(),
                                         kv.second.real(), kv.second.imag()});
    if (a < 0 || a >= DN || b < 0 || b >= DN) continue;
    const double uu = u[a * DN + b];
    const double row1 = 1.0 / (EPS1 + (uu - du) * (EPS2 - EPS1));
    const double row2 = 1.0 / (EPS1 + (uu + du) * (EPS2 - EPS1));
    const complex<double> prod = kv.second * (fv * (row1 - row2) / (2 * du));
    grad[a * DN + b] += prod.real();
  }
  w.rec("design_dft", rec_design);
  w.rec("grad_u", grad);

  /* central differences of J on the reference core */
  std::vector<int> order(DN * DN);
  for (int k = 0; k < DN * DN; k++)
    order[k] = k;
  std::sort(order.begin(), order.end(), [&](int x, int y) { return std::fabs(grad[x]) > std::fabs(grad[y]); });
  const double h = 1e-3;
  std::vector<double> fd;
  for (int q = 0; q < 4; q++) {
    const int k = order[q], a = k / DN, b = k % DN;
    std::vector<double> ep = eps, em = eps;
    ep[(DI0 + a) * (NY + 1) + DJ0 + b] = EPS1 + (u[k] + h) * (EPS2 - EPS1);
    em[(DI0 + a) * (NY + 1) + DJ0 + b] = EPS1 + (u[k] - h) * (EPS2 - EPS1);
    fd.push_back(k);
    fd.push_back((forward_J(ep) - forward_J(em)) / (2 * h));
  }
  w.rec("fd_pixels", fd);
  std::vector<double> dp(DN * DN);
  for (double &x : dp)
    x = uni(rng) - 0.5;
  const double hs = 1e-3;
  std::vector<double> ep = eps, em = eps;
  for (int k = 0; k < DN * DN; k++) {
    const int a = k / DN, b = k % DN;
    ep[(DI0 + a) * (NY + 1) + DJ0 + b] = EPS1 + (u[k] + hs * dp[k]) * (EPS2 - EPS1);
    em[(DI0 + a) * (NY + 1) + DJ0 + b] = EPS1 + (u[k] - hs * dp[k]) * (EPS2 - EPS1);
  }
  w.rec("dp", dp);
  w.scalar("fd_directional", (forward_J(ep) - forward_J(em)) / (2 * hs));
}
#endif

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
  else if (cs == "vec3d_full_trunc")
    case_vec3d_full_trunc(w, steps > 0 ? steps : 600);
  else if (cs == "disp3d_full_trunc")
    case_disp3d_full_trunc(w, steps > 0 ? steps : 384);
  else if (cs == "disp3d_cube")
    case_disp3d_cube(w, steps > 0 ? steps : 3000);
  else if (cs == "disp3d_small")
    case_disp3d(w, 20, 18, 16, 20.0, 0.25, steps > 0 ? steps : 600, 7, true, 1);
  else if (cs == "known")
    case_known(w);
  else if (cs == "py_tm2d")
    case_py_tm2d(w);
  else if (cs == "py_disp3d")
    case_py_disp3d(w);
  else if (cs == "aniso_te2d")
    case_aniso_te2d(w, steps > 0 ? steps : 400);
  else if (cs == "aniso3d")
    case_aniso3d(w, steps > 0 ? steps : 200);
  else if (cs == "offdiag_te2d")
    case_offdiag_te2d(w, steps > 0 ? steps : 400);
  else if (cs == "aniso_bloch2d")
    case_aniso_bloch2d(w, steps > 0 ? steps : 300);
  else if (cs == "py_aniso_te2d")
    case_py_aniso_te2d(w);
  else if (cs == "py_aniso3d")
    case_py_aniso3d(w);
  else if (cs == "aniso1d")
    case_aniso1d(w, steps > 0 ? steps : 400);
  else if (cs == "n2f_tm2d")
    case_n2f(w, D2, Ez, Hx, steps > 0 ? steps : 2800);
  else if (cs == "n2f_te2d")
    case_n2f(w, D2, Ex, Hz, steps > 0 ? steps : 2800);
  else if (cs == "n2f3d")
    case_n2f(w, D3, Ez, Hx, steps > 0 ? steps : 900);
  else if (cs == "py_ldos")
    case_py_ldos(w);
  else if (cs == "py_matgrid")
    case_py_matgrid(w);
  else if (cs == "py_energy")
    case_py_energy(w);
  else if (cs == "py_force")
    case_py_force(w);
  else if (cs == "py_n2f")
    case_py_n2f(w);
  else if (cs == "n2f_periodic2d")
    case_n2f_periodic2d(w, steps > 0 ? steps : 1600);
#ifndef MEEP_GB300
  else if (cs == "adjoint_tm2d")
    case_adjoint_tm2d(w);
#endif
  else {
    fprintf(stderr, "unknown case %s\n", cs.c_str());
    return 2;
  }
  return 0;
}
