// Implementation of the drop-in meep:: API (include/meep_gb300/meep.hpp) over
// the C ABI in mfd.h.
//
// Host-side setup follows the reference's semantics so that the engine sees the
// same inputs the reference's chunks would hold:
//   material arrays   structure_chunk::set_chi1inv   src/anisotropic_averaging.cpp:211-324
//                     structure_chunk::set_conductivity src/structure.cpp:868-905
//                     structure_chunk::add_susceptibility src/anisotropic_averaging.cpp:330-417
//   component set     fields::_require_component     src/fields.cpp:552-572
//   source points     fields::add_volume_source      src/sources.cpp:223-312, 463-489
//   monitor points    fields::loop_in_chunks         src/loop_in_chunks.cpp:283-540
//                     compute_boundary_weights       src/loop_in_chunks.cpp:245-281
//   DFT setup         fields::add_dft / add_dft_flux src/dft.cpp:175-235, 602-652
//   interpolation     grid_volume::interpolate       src/vec.cpp:527-612
// The whole cell is one chunk here, so loop_in_chunks reduces to its
// single-chunk case (identity symmetry, no periodic images).
#include <meep.hpp>

#include <algorithm>
#include <cstdarg>
#include <cstring>
#include <map>

#include "mfd.h"
#include "subpixel.hpp"

namespace meep {

int verbosity = 1;

void abort(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  char buf[1024];
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  throw std::runtime_error(std::string("meep: ") + buf);
}

void master_printf(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vprintf(fmt, ap);
  va_end(ap);
}

const char *component_name(component c) {
  static const char *names[] = {"ex", "ey", "er", "ep", "ez", "hx", "hy", "hr", "hp", "hz",
                                "dx", "dy", "dr", "dp", "dz", "bx", "by", "br", "bp", "bz",
                                "eps", "mu", "none"};
  return names[c];
}

static int mfd_comp(component c) {
  int t = type(c);
  direction d = component_direction(c);
  if (d > Z) meep::abort("cylindrical components are not supported");
  return 3 * t + int(d);
}

static void chk(int status) {
  if (status != 0) throw std::runtime_error(mfd_last_error());
}

/* ---------------------------------------------------------- geometry */
volume::volume(const vec &vec1, const vec &vec2) : dim(vec1.dim), min_corner(vec1.dim), max_corner(vec1.dim) {
  LOOP_OVER_DIRECTIONS(dim, d) {
    min_corner.set_direction(d, std::min(vec1.in_direction(d), vec2.in_direction(d)));
    max_corner.set_direction(d, std::max(vec1.in_direction(d), vec2.in_direction(d)));
  }
}

grid_volume::grid_volume(ndim td, double ta, int na, int nb, int nc) : io(td), origin(td) {
  dim = td;
  a = ta;
  inva = 1.0 / ta;
  num[0] = na;
  num[1] = nb;
  num[2] = nc;
  set_origin(zero_ivec(dim));
}

void grid_volume::set_origin(const ivec &o) {
  io = o;
  origin = operator[](io);
}

ivec grid_volume::big_corner() const {
  ivec r = io;
  LOOP_OVER_DIRECTIONS(dim, d) r.t[d] += 2 * num_direction(d);
  return r;
}

ivec grid_volume::iyee_shift(component c) const {
  ivec out = zero_ivec(dim);
  LOOP_OVER_DIRECTIONS(dim, d) {
    if (c == Dielectric || c == Permeability ||
        ((is_electric(c) || is_D(c)) && d == component_direction(c)) ||
        ((is_magnetic(c) || is_B(c)) && d != component_direction(c)))
      out.set_direction(d, 1);
  }
  return out;
}

ivec grid_volume::icenter() const {
  ivec r = io;
  LOOP_OVER_DIRECTIONS(dim, d) {
    int v = num_direction(d);
    r.t[d] += v - (v >= 0 ? v : -v) % 2;
  }
  return r;
}

bool grid_volume::owns(const ivec &p) const {
  LOOP_OVER_DIRECTIONS(dim, d) {
    int o = p.in_direction(d) - io.in_direction(d);
    if (!(o > 0 && o <= 2 * num_direction(d))) return false;
  }
  return true;
}

double grid_volume::boundary_location(boundary_side b, direction d) const {
  int i = io.in_direction(d) + (b == High ? 2 * num_direction(d) : 0);
  return i * (0.5 * inva);
}

size_t grid_volume::ntot() const {
  size_t n = 1;
  LOOP_OVER_DIRECTIONS(dim, d) n *= (size_t)(num_direction(d) + 1);
  return n;
}

grid_volume volone(double zsize, double a) { return grid_volume(D1, a, 0, 0, (int)(zsize * a + 0.5)); }
grid_volume vol1d(double zsize, double a) { return volone(zsize, a); }
grid_volume voltwo(double xsize, double ysize, double a) {
  return grid_volume(D2, a, (xsize == 0) ? 1 : (int)(xsize * a + 0.5),
                     (ysize == 0) ? 1 : (int)(ysize * a + 0.5), 0);
}
grid_volume vol2d(double xsize, double ysize, double a) { return voltwo(xsize, ysize, a); }
grid_volume vol3d(double xsize, double ysize, double zsize, double a) {
  return grid_volume(D3, a, (xsize == 0) ? 1 : (int)(xsize * a + 0.5),
                     (ysize == 0) ? 1 : (int)(ysize * a + 0.5),
                     (zsize == 0) ? 1 : (int)(zsize * a + 0.5));
}

symmetry identity() { return symmetry(); }

boundary_region pml(double thickness, direction d, boundary_side side, double Rasymptotic,
                    double mean_stretch) {
  return boundary_region(boundary_region::PML, thickness, Rasymptotic, mean_stretch, d, side);
}
boundary_region pml(double thickness, direction d, double Rasymptotic, double mean_stretch) {
  return pml(thickness, d, Low, Rasymptotic, mean_stretch) +
         pml(thickness, d, High, Rasymptotic, mean_stretch);
}
boundary_region pml(double thickness, double Rasymptotic, double mean_stretch) {
  boundary_region r;
  for (int id = 0; id < 3; ++id)
    r = r + pml(thickness, (direction)id, Rasymptotic, mean_stretch);
  return r;
}

/* Subpixel averaging through the shared host/device routine (subpixel.hpp):
   the pixel as [lo, hi] in x, y, z order, chi1p1 called with a vec of the
   grid's dimension. */
static int subpixel_dim(ndim dim) {
  if (dim == D1) return 1;
  if (dim == D2) return 2;
  if (dim == D3) return 3;
  meep::abort("subpixel averaging in cylindrical coordinates is not supported by the GB300 engine");
}

static void volume_box(const volume &v, double lo[3], double hi[3]) {
  for (int d = 0; d < 3; d++) {
    lo[d] = hi[d] = 0.0;
  }
  LOOP_OVER_DIRECTIONS(v.dim, d) {
    lo[d] = v.in_direction_min(d);
    hi[d] = v.in_direction_max(d);
  }
}

namespace {
struct ChiOf {
  material_function *m;
  field_type ft;
  ndim dim;
  double operator()(const double p[3]) const {
    vec r(dim);
    LOOP_OVER_DIRECTIONS(dim, d) r.set_direction(d, p[d]);
    return m->chi1p1(ft, r);
  }
};
} // namespace

vec material_function::normal_vector(field_type ft, const volume &v) {
  double lo[3], hi[3], g[3];
  volume_box(v, lo, hi);
  mgb_subpixel::normal_vector(subpixel_dim(v.dim), lo, hi, mgb_subpixel::sphere_quadrature(),
                              ChiOf{this, ft, v.dim}, g);
  vec out(v.dim);
  LOOP_OVER_DIRECTIONS(v.dim, d) out.set_direction(d, g[d]);
  return out;
}

void material_function::eff_chi1inv_row(component c, double chi1inv_row[3], const volume &v,
                                        double tol, int maxeval) {
  double lo[3], hi[3];
  volume_box(v, lo, hi);
  mgb_subpixel::eff_chi1inv_row(subpixel_dim(v.dim), component_direction(c) % 3, lo, hi, tol, maxeval,
                                mgb_subpixel::sphere_quadrature(), ChiOf{this, type(c), v.dim},
                                chi1inv_row);
}

std::vector<double> linspace(double freq_min, double freq_max, size_t Nfreq) {
  std::vector<double> freq(Nfreq);
  for (size_t i = 0; i < Nfreq; ++i)
    freq[i] = freq_min + (Nfreq <= 1 ? 0.0 : (freq_max - freq_min) * i / (Nfreq - 1));
  return freq;
}

/* Dense component-grid helpers: point k of component c along direction d sits
   at ivec io + shift + 2k; dense index with x slowest, last direction fastest. */
struct Dense {
  ndim dim;
  int n[3];     // cells per X,Y,Z (0 absent)
  int ext[3];   // points per X,Y,Z (1 absent)
  ivec io;
  explicit Dense(const grid_volume &gv) : dim(gv.dim), io(gv.little_corner()) {
    for (int d = 0; d < 3; d++) {
      n[d] = 0;
      ext[d] = 1;
    }
    LOOP_OVER_DIRECTIONS(gv.dim, d) {
      n[d] = gv.num_direction(d);
      ext[d] = n[d] + 1;
    }
  }
  size_t count() const { return (size_t)ext[0] * ext[1] * ext[2]; }
  int64_t index(const int k[3]) const { return ((int64_t)k[0] * ext[1] + k[1]) * ext[2] + k[2]; }
  void coords(int64_t di, int k[3]) const {
    k[2] = int(di % ext[2]);
    di /= ext[2];
    k[1] = int(di % ext[1]);
    k[0] = int(di / ext[1]);
  }
  // k of an ivec location for component c (no range check)
  void kof(const grid_volume &gv, component c, const ivec &p, int k[3]) const {
    ivec sh = gv.iyee_shift(c);
    k[0] = k[1] = k[2] = 0;
    LOOP_OVER_DIRECTIONS(dim, d) k[d] = (p.in_direction(d) - io.in_direction(d) - sh.in_direction(d)) / 2;
  }
  ivec iloc(const grid_volume &gv, component c, const int k[3]) const {
    ivec p = io + gv.iyee_shift(c);
    LOOP_OVER_DIRECTIONS(dim, d) p.t[d] += 2 * k[d];
    return p;
  }
  template <class F> void for_each(F fn) const {
    int k[3];
    for (k[0] = 0; k[0] < ext[0]; k[0]++)
      for (k[1] = 0; k[1] < ext[1]; k[1]++)
        for (k[2] = 0; k[2] < ext[2]; k[2]++)
          fn(k, index(k));
  }
  // same, with the slowest direction spread over OpenMP threads (for
  // material functions that declare themselves thread-safe)
  template <class F> void for_each_parallel(F fn) const {
#pragma omp parallel for schedule(dynamic, 1)
    for (int k0 = 0; k0 < ext[0]; k0++) {
      int k[3];
      k[0] = k0;
      for (k[1] = 0; k[1] < ext[1]; k[1]++)
        for (k[2] = 0; k[2] < ext[2]; k[2]++)
          fn(k, index(k));
    }
  }
};

/* ----------------------------------------------------------- structure */
struct PoleSpec {
  double omega0, gamma;
  bool drude;
  std::vector<double> sigma[3]; // dense per E component direction (empty = absent)
};

struct MatGridRec {
  double center[3], size[3], beta, eta, eps1[3], eps2[3];
  int n[3];
  std::vector<double> u;
};

struct structure::impl {
  std::vector<double> chi1inv[3][3]; // [E component direction][row entry direction]
  std::vector<double> cond[2][3];    // [0 = D, 1 = B][direction]
  std::vector<PoleSpec> poles;       // in add order
  std::vector<MatGridRec> matgrids;  // in add order
  bool engine_created = false;       // materials were handed to an engine
};

static volume dV(const grid_volume &gv, const ivec &here, double diameter = 1.0) {
  const double hinva = 0.5 * gv.inva * diameter;
  const vec h = gv[here];
  volume out(gv.dim);
  LOOP_OVER_DIRECTIONS(gv.dim, d) {
    out.set_direction_max(d, h.in_direction(d) + hinva);
    out.set_direction_min(d, h.in_direction(d) - hinva);
  }
  return out;
}

static vec loop_loc(const grid_volume &gv, const ivec &p) {
  // IVEC_LOOP_LOC: (0.5*is + i)*inva, which equals (0.5*p)*inva exactly
  vec r(gv.dim);
  LOOP_OVER_DIRECTIONS(gv.dim, d) r.set_direction(d, (0.5 * p.in_direction(d)) * gv.inva);
  return r;
}

structure::structure(const grid_volume &thegv, material_function &eps, const boundary_region &br_,
                     const symmetry &s, int num_chunks, double Courant_, bool use_aa, double tol,
                     int maxeval)
    : gv(thegv), user_volume(thegv), a(thegv.a), Courant(Courant_), dt(Courant_ / thegv.a), br(br_),
      d(new impl) {
  (void)s;
  (void)num_chunks;
  set_materials(eps, use_aa, tol, maxeval);
}

static material_function *new_simple(double f(const vec &)) { return new simple_material_function(f); }

structure::structure(const grid_volume &thegv, double epsf(const vec &), const boundary_region &br_,
                     const symmetry &s, int num_chunks, double Courant_, bool use_aa, double tol,
                     int maxeval)
    : gv(thegv), user_volume(thegv), a(thegv.a), Courant(Courant_), dt(Courant_ / thegv.a), br(br_),
      d(new impl) {
  (void)s;
  (void)num_chunks;
  std::unique_ptr<material_function> m(new_simple(epsf));
  set_materials(*m, use_aa, tol, maxeval);
}

structure::~structure() {}

void structure::set_materials(material_function &mat, bool use_aa, double tol, int maxeval) {
  set_epsilon(mat, use_aa, tol, maxeval);
  if (mat.has_mu()) meep::abort("mu != 1 is not supported by the GB300 engine");
  const component dcs[6] = {Dx, Dy, Dz, Bx, By, Bz};
  for (component c : dcs)
    if (gv.has_field(c) && mat.has_conductivity(c)) set_conductivity(c, mat);
  const component ecs[6] = {Ex, Ey, Ez, Hx, Hy, Hz};
  for (component c : ecs)
    if (gv.has_field(c) && (mat.has_chi3(c) || mat.has_chi2(c)))
      meep::abort("nonlinear susceptibilities are not supported by the GB300 engine");
}

// set_chi1inv: the diagonal entry from the pixel centred at the point, the
// off-diagonal entries from the pixel shifted half a cell back along the
// component direction; entries equal to the identity everywhere are dropped
// (src/anisotropic_averaging.cpp:211-324).
void structure::set_epsilon(material_function &mat, bool use_aa, double tol, int maxeval) {
  if (!use_aa) maxeval = 0;
  Dense dn(gv);
  const component ecs[3] = {Ex, Ey, Ez};
  for (component c : ecs) {
    if (!gv.has_field(c)) continue;
    int dc = component_direction(c);
    std::vector<double> arr[3];
    bool trivial[3] = {true, true, true};
    for (int q = 0; q < 3; q++)
      arr[q].assign(dn.count(), 0.0);
    ivec shift1(gv.dim, 0);
    shift1.set_direction(direction(dc), 1);
    // bulk evaluation first (two pixels per point, in batches), else pixel
    // by pixel through eff_chi1inv_row
    bool bulk = true;
    {
      const size_t npts = dn.count(), B = size_t(1) << 18;
      std::vector<double> lo, hi, rows;
      for (size_t p0 = 0; p0 < npts && bulk; p0 += B) {
        const size_t nb = std::min(B, npts - p0);
        lo.resize(6 * nb);
        hi.resize(6 * nb);
        rows.resize(6 * nb);
        for (size_t j = 0; j < nb; j++) {
          int k[3];
          dn.coords((int64_t)(p0 + j), k);
          const ivec here = dn.iloc(gv, c, k);
          volume_box(dV(gv, here), &lo[6 * j], &hi[6 * j]);
          volume_box(dV(gv, here - shift1), &lo[6 * j + 3], &hi[6 * j + 3]);
        }
        if (!mat.eff_chi1inv_rows(c, 2 * nb, lo.data(), hi.data(), tol, maxeval, rows.data())) {
          bulk = false;
          break;
        }
        for (size_t j = 0; j < nb; j++)
          for (int q = 0; q < 3; q++)
            arr[q][p0 + j] = (q == dc) ? rows[6 * j + q] : rows[6 * j + 3 + q];
      }
    }
    auto body = [&](const int k[3], int64_t di) {
      ivec here = dn.iloc(gv, c, k);
      double row[3], row_off[3];
      mat.eff_chi1inv_row(c, row, dV(gv, here), tol, maxeval);
      mat.eff_chi1inv_row(c, row_off, dV(gv, here - shift1), tol, maxeval);
      for (int q = 0; q < 3; q++)
        arr[q][di] = (q == dc) ? row[q] : row_off[q];
    };
    if (!bulk) {
      if (mat.is_thread_safe()) dn.for_each_parallel(body);
      else dn.for_each(body);
    }
    for (int q = 0; q < 3; q++)
      for (double v : arr[q])
        if (v != (q == dc ? 1.0 : 0.0)) {
          trivial[q] = false;
          break;
        }
    for (int q = 0; q < 3; q++) {
      if (q != dc && trivial[q]) arr[q].clear();
      d->chi1inv[dc][q] = std::move(arr[q]);
    }
    if (trivial[0] && trivial[1] && trivial[2]) d->chi1inv[dc][dc].clear();
  }
}

void structure::set_conductivity(component c, material_function &C) {
  if (!gv.has_field(c)) return;
  direction cd = component_direction(c);
  if (cd > Z) meep::abort("cylindrical components are not supported");
  int which = is_H_or_B(c) ? 1 : 0;
  component cC = direction_component(which ? Bx : Dx, cd);
  Dense dn(gv);
  std::vector<double> arr(dn.count(), 0.0);
  bool trivial = true;
  const std::vector<double> *multby = nullptr;
  if (is_electric(c) && !d->chi1inv[cd][cd].empty()) multby = &d->chi1inv[cd][cd];
  if (is_magnetic(c)) meep::abort("magnetic conductivity with mu is not supported");
  dn.for_each([&](const int k[3], int64_t di) {
    vec here = loop_loc(gv, dn.iloc(gv, cC, k));
    double v = C.conductivity(c, here);
    if (multby) v = v * (*multby)[di];
    arr[di] = v;
    if (v != 0.0) trivial = false;
  });
  d->cond[which][cd] = trivial ? std::vector<double>() : arr;
}

void structure::set_epsilon(double epsf(const vec &), bool use_aa, double tol, int maxeval) {
  std::unique_ptr<material_function> m(new_simple(epsf));
  set_epsilon(*m, use_aa, tol, maxeval);
}

std::complex<double> structure::get_chi1inv(component c, direction dd, const ivec &origloc, double frequency,
                                            bool parallel) const {
  (void)parallel;
  if (frequency != 0) meep::abort("frequency-dependent chi1inv is not supported by the GB300 engine");
  if (!gv.owns(origloc)) return 0.0;
  const direction cd = component_direction(c);
  const double ident = dd == cd ? 1.0 : 0.0;
  if (!is_electric(c) || cd > Z || dd > Z) return ident;
  const std::vector<double> &arr = d->chi1inv[cd][dd];
  if (arr.empty()) return ident;
  Dense dn(gv);
  int k[3];
  dn.kof(gv, c, origloc, k);
  return arr[dn.index(k)];
}

void structure::set_conductivity(component c, double Cfunc(const vec &)) {
  simple_material_function m(Cfunc);
  set_conductivity(c, m);
}

// add_susceptibility: sigma rows per E component; diagonal from the point,
// off-diagonal from the point shifted by -1 along the component direction
// (src/anisotropic_averaging.cpp:330-417).
void structure::add_susceptibility(material_function &sigma, field_type ft,
                                   const susceptibility &sus) {
  if (ft != E_stuff) meep::abort("only electric susceptibilities are supported by the GB300 engine");
  const lorentzian_susceptibility *lz = dynamic_cast<const lorentzian_susceptibility *>(&sus);
  if (!lz) meep::abort("only Lorentzian/Drude susceptibilities are supported by the GB300 engine");
  PoleSpec ps;
  ps.omega0 = lz->omega_0;
  ps.gamma = lz->gamma;
  ps.drude = lz->no_omega_0_denominator;
  Dense dn(gv);
  const component ecs[3] = {Ex, Ey, Ez};
  for (component c : ecs) {
    if (!gv.has_field(c)) continue;
    int dc = component_direction(c);
    ivec unit(gv.dim, 0);
    unit.set_direction(direction(dc), 1);
    vec shift1 = gv[unit];
    std::vector<double> arr(dn.count(), 0.0);
    bool trivial = true;
    dn.for_each([&](const int k[3], int64_t di) {
      vec here = loop_loc(gv, dn.iloc(gv, c, k));
      double row[3], row_off[3];
      sigma.sigma_row(c, row, here);
      sigma.sigma_row(c, row_off, here - shift1);
      for (int q = 0; q < 3; q++)
        if (q != dc && row_off[q] != 0.0)
          meep::abort("anisotropic susceptibilities are not supported by the GB300 engine");
      arr[di] = row[dc];
      if (row[dc] != 0.0) trivial = false;
    });
    if (!trivial) ps.sigma[dc] = std::move(arr);
  }
  d->poles.push_back(std::move(ps));
}

void structure::add_susceptibility(double sigma(const vec &), field_type ft,
                                   const susceptibility &sus) {
  simple_material_function m(sigma);
  add_susceptibility(m, ft, sus);
}

void structure::add_material_grid(const double center[3], const double size[3], const int n[3],
                                  const double *weights, double beta, double eta, const double eps1[3],
                                  const double eps2[3]) {
  if (!center || !size || !n || !weights || !eps1 || !eps2) meep::abort("null material grid argument");
  if (n[0] < 1 || n[1] < 1 || n[2] < 1) meep::abort("material grid sizes must be at least 1");
  if (d->engine_created) meep::abort("material grids must be added before the fields are stepped or monitored");
  MatGridRec m;
  for (int q = 0; q < 3; q++) {
    m.center[q] = center[q];
    m.size[q] = size[q];
    m.n[q] = n[q];
    m.eps1[q] = eps1[q];
    m.eps2[q] = eps2[q];
  }
  m.beta = beta;
  m.eta = eta;
  m.u.assign(weights, weights + (size_t)n[0] * n[1] * n[2]);
  d->matgrids.push_back(std::move(m));
}

/* ------------------------------------------------------------- sources */
gaussian_src_time::gaussian_src_time(double f, double fw, double s) : explicit_window(false) {
  freq = f;
  width = 1.0 / fw;
  peak_time = width * s;
  cutoff = width * s;
  fwidth = std::sqrt(-2.0 * std::log(1e-7)) / (width * pi);
  while (std::exp(-cutoff * cutoff / (2 * width * width)) < 1e-100)
    cutoff *= 0.9;
  cutoff = float(cutoff);
  p[0] = f;
  p[1] = fw;
  p[2] = s;
}

gaussian_src_time::gaussian_src_time(double f, double w, double st, double et) : explicit_window(true) {
  freq = f;
  width = w;
  peak_time = 0.5 * (st + et);
  cutoff = (et - st) * 0.5;
  fwidth = std::sqrt(-2.0 * std::log(1e-7)) / (width * pi);
  while (std::exp(-cutoff * cutoff / (2 * width * width)) < 1e-100)
    cutoff *= 0.9;
  cutoff = float(cutoff);
  p[0] = f;
  p[1] = w;
  p[2] = st;
  p[3] = et;
}

continuous_src_time::continuous_src_time(std::complex<double> f, double w, double st, double et,
                                         double s)
    : freq(f), width(w), start_time(float(st)), end_time(float(et)), slowness(s) {
  p[0] = f.real();
  p[1] = f.imag();
  p[2] = w;
  p[3] = st;
  p[4] = et;
  p[5] = s;
}

/* --------------------------------------------------------------- fields */
struct PendingSource {
  int c;     // mfd component
  int src;   // index into srcs
  std::vector<int64_t> idx;
  std::vector<std::complex<double>> amp;
};

struct fields::impl {
  mfd_sim *sim = nullptr;
  std::vector<std::unique_ptr<src_time>> srcs;
  std::vector<PendingSource> pending;
  int components = 0;
  std::vector<std::unique_ptr<dft_chunk>> chunks; // owned dft chunks
  std::vector<dft_flux *> fluxes;
  bool real_fields = false;
  // Bloch-periodic boundaries (use_bloch): periodic directions, k, and
  // eikna = exp(2 pi i k L) as the engine computes it
  int periodic[3] = {0, 0, 0};
  double kvec[3] = {0, 0, 0};
  std::complex<double> eikna[3] = {{1, 0}, {1, 0}, {1, 0}};
  bool complex_fields() const {
    for (int q = 0; q < 3; q++)
      if (periodic[q] && kvec[q] != 0.0) return true;
    return false;
  }
  // cache of downloaded fields for get_field (real and imaginary parts)
  int64_t cache_t[20];
  std::vector<double> cache[20], cache_im[20];
  impl() {
    for (int i = 0; i < 20; i++)
      cache_t[i] = -1;
  }
  ~impl() {
    if (sim) mfd_destroy(sim);
  }
};

fields::fields(structure *s_, double m, double beta, bool zcyl, int tdb, int teh)
    : t(0), dt(s_->dt), a(s_->a), gv(s_->gv), user_volume(s_->user_volume), s(s_), d(new impl) {
  (void)zcyl;
  (void)tdb;
  (void)teh;
  if (m != 0 || beta != 0) meep::abort("m != 0 / beta != 0 are not supported by the GB300 engine");
}

fields::~fields() {}

void fields::use_real_fields() {
  if (d->complex_fields()) meep::abort("Can't use real fields with bloch boundary conditions!\n");
  d->real_fields = true;
}

// fields::use_bloch (src/boundaries.cpp:90-117): periodic boundaries along d
// with Bloch wavevector k (units of 2 pi / a); a nonzero k needs complex
// fields
void fields::use_bloch(direction dd, double k) {
  if (d->sim) meep::abort("use_bloch must be called before the first step");
  if (dd > Z) meep::abort("use_bloch along a non-Cartesian direction is not supported");
  d->periodic[dd] = 1;
  d->kvec[dd] = k;
  const double L = gv.num_direction(dd);
  if (k * L == 0.5 * a) d->eikna[dd] = -1.0;
  else d->eikna[dd] = std::exp(std::complex<double>(0.0, 1.0) * std::complex<double>(k, 0.0) * ((2 * pi / a) * L));
  if (d->real_fields && k != 0.0) meep::abort("Can't use real fields with bloch boundary conditions!\n");
}

void fields::use_bloch(const vec &k) {
  LOOP_OVER_DIRECTIONS(gv.dim, dd) use_bloch(dd, k.in_direction(dd));
}

static bool is_like(ndim dim, component c1, component c2) {
  if (dim != D2) return true;
  auto tm = [](component c) {
    return c == Hx || c == Hy || c == Bx || c == By || c == Ez || c == Dz;
  };
  return !(tm(c1) ^ tm(c2));
}

// _require_component (src/fields.cpp:552-572): allocate every like component
static int require_components(const grid_volume &gv, component c, int mask) {
  if (!gv.has_field(c)) meep::abort("cannot require a %s component in this grid", component_name(c));
  for (int ci = 0; ci < 20; ci++) {
    component ca = component(ci);
    if (gv.has_field(ca) && is_like(gv.dim, c, ca)) mask |= 1 << mfd_comp(ca);
  }
  return mask;
}

static void ensure_engine(fields &f) {
  fields::impl &I = *f.d;
  if (I.sim) return;
  if (!I.components) meep::abort("allocate field components (by adding sources) before stepping");
  const grid_volume &gv = f.gv;
  mfd_grid g;
  std::memset(&g, 0, sizeof(g));
  g.dim = gv.dim == D1 ? 1 : gv.dim == D2 ? 2 : 3;
  if (gv.dim == Dcyl) meep::abort("cylindrical coordinates are not supported");
  LOOP_OVER_DIRECTIONS(gv.dim, dd) {
    g.n[dd] = gv.num_direction(dd);
    g.io[dd] = gv.little_corner().in_direction(dd);
  }
  g.a = gv.a;
  g.courant = f.s->Courant;
  for (const auto &pt : f.s->br.parts) {
    if (pt.kind != boundary_region::PML) continue;
    if (pt.d > Z) continue;
    bool present = false;
    LOOP_OVER_DIRECTIONS(gv.dim, dd) present = present || dd == pt.d;
    if (!present || gv.num_direction(pt.d) <= 1) continue;
    int side = pt.side == Low ? 0 : 1;
    g.pml_thickness[pt.d][side] = pt.thickness;
    g.pml_R[pt.d][side] = pt.Rasymptotic;
    g.pml_stretch[pt.d][side] = pt.mean_stretch;
  }
  g.precision = sizeof(realnum) == 8 ? 64 : 32;
  g.components = I.components;
  chk(mfd_create(&g, &I.sim));
  if (I.periodic[0] || I.periodic[1] || I.periodic[2]) chk(mfd_set_bloch(I.sim, I.periodic, I.kvec));
  structure::impl &S = *f.s->d;
  for (int dc = 0; dc < 3; dc++)
    for (int q = 0; q < 3; q++)
      if (!S.chi1inv[dc][q].empty() && ((I.components >> (3 * MFD_E + dc)) & 1))
        chk(mfd_set_chi1inv(I.sim, 3 * MFD_E + dc, q, S.chi1inv[dc][q].data()));
  for (int w = 0; w < 2; w++)
    for (int dc = 0; dc < 3; dc++)
      if (!S.cond[w][dc].empty()) {
        int c = 3 * (w ? MFD_B : MFD_D) + dc;
        if ((I.components >> c) & 1) chk(mfd_set_conductivity(I.sim, c, S.cond[w][dc].data()));
      }
  for (const PoleSpec &ps : S.poles) {
    const double *sg[3] = {nullptr, nullptr, nullptr};
    for (int q = 0; q < 3; q++)
      if (!ps.sigma[q].empty() && ((I.components >> (3 * MFD_E + q)) & 1)) sg[q] = ps.sigma[q].data();
    chk(mfd_add_lorentzian(I.sim, MFD_E, ps.omega0, ps.gamma, ps.drude ? 1 : 0, sg));
  }
  for (const MatGridRec &m : S.matgrids)
    chk(mfd_add_material_grid(I.sim, m.center, m.size, m.n, m.u.data(), m.beta, m.eta, m.eps1, m.eps2, nullptr));
  S.engine_created = true;
  std::vector<int> ids;
  for (const auto &st : I.srcs) {
    int id = -1;
    if (st->kind() == 0) {
      const gaussian_src_time *gs = static_cast<const gaussian_src_time *>(st.get());
      if (gs->explicit_window)
        chk(mfd_add_gaussian_src(I.sim, gs->p[0], gs->p[1], gs->p[2], gs->p[3], 1,
                                 st->is_integrated, &id));
      else
        chk(mfd_add_gaussian_src(I.sim, gs->p[0], gs->p[1], gs->p[2], 0, 0, st->is_integrated, &id));
    }
    else {
      chk(mfd_add_continuous_src(I.sim, st->p[0], st->p[1], st->p[2], st->p[3], st->p[4], st->p[5],
                                 st->is_integrated, &id));
    }
    ids.push_back(id);
  }
  for (const PendingSource &ps : I.pending) {
    std::vector<double> amp(2 * ps.amp.size());
    for (size_t j = 0; j < ps.amp.size(); j++) {
      amp[2 * j] = ps.amp[j].real();
      amp[2 * j + 1] = ps.amp[j].imag();
    }
    chk(mfd_add_source_points(I.sim, ps.c, ids[ps.src], ps.idx.size(), ps.idx.data(), amp.data()));
  }
}

/* ----------------------------------------------------- loop_in_chunks */
struct LoopBox {
  bool empty = true;
  ivec is, ie;                // in cgrid ivec coordinates
  vec s0, s1, e0, e1;         // per-direction weights (absent directions 1)
  double dV0 = 1.0;
};

static ivec vec2diel_floor(const vec &pt, double a, const ivec &equal_shift) {
  ivec ipt(pt.dim);
  LOOP_OVER_DIRECTIONS(pt.dim, d) {
    ipt.set_direction(d, 1 + 2 * int(std::floor(pt.in_direction(d) * a - .5)));
    if (ipt.in_direction(d) == pt.in_direction(d))
      ipt.set_direction(d, ipt.in_direction(d) + equal_shift.in_direction(d));
  }
  return ipt;
}
static ivec vec2diel_ceil(const vec &pt, double a, const ivec &equal_shift) {
  ivec ipt(pt.dim);
  LOOP_OVER_DIRECTIONS(pt.dim, d) {
    ipt.set_direction(d, 1 + 2 * int(std::ceil(pt.in_direction(d) * a - .5)));
    if (ipt.in_direction(d) == pt.in_direction(d))
      ipt.set_direction(d, ipt.in_direction(d) + equal_shift.in_direction(d));
  }
  return ipt;
}

static void compute_boundary_weights(const grid_volume &gv, const volume &where, ivec &is, ivec &ie,
                                     bool snap_empty_dimensions, vec &s0, vec &e0, vec &s1, vec &e1) {
  LOOP_OVER_DIRECTIONS(gv.dim, d) {
    double w0, w1;
    w0 = 1. - where.in_direction_min(d) * gv.a + 0.5 * is.in_direction(d);
    w1 = 1. + where.in_direction_max(d) * gv.a - 0.5 * ie.in_direction(d);
    if (ie.in_direction(d) >= is.in_direction(d) + 3 * 2) {
      s0.set_direction(d, w0 * w0 / 2);
      s1.set_direction(d, 1 - (1 - w0) * (1 - w0) / 2);
      e0.set_direction(d, w1 * w1 / 2);
      e1.set_direction(d, 1 - (1 - w1) * (1 - w1) / 2);
    }
    else if (ie.in_direction(d) == is.in_direction(d) + 2 * 2) {
      s0.set_direction(d, w0 * w0 / 2);
      s1.set_direction(d, 1 - (1 - w0) * (1 - w0) / 2 - (1 - w1) * (1 - w1) / 2);
      e0.set_direction(d, w1 * w1 / 2);
      e1.set_direction(d, s1.in_direction(d));
    }
    else if (where.in_direction_min(d) == where.in_direction_max(d)) {
      if (snap_empty_dimensions) {
        if (w0 > w1) ie.set_direction(d, is.in_direction(d));
        else is.set_direction(d, ie.in_direction(d));
        w0 = w1 = 1.0;
      }
      s0.set_direction(d, w0);
      s1.set_direction(d, w1);
      e0.set_direction(d, w1);
      e1.set_direction(d, w0);
    }
    else if (ie.in_direction(d) == is.in_direction(d) + 1 * 2) {
      s0.set_direction(d, w0 * w0 / 2 - (1 - w1) * (1 - w1) / 2);
      e0.set_direction(d, w1 * w1 / 2 - (1 - w0) * (1 - w0) / 2);
      s1.set_direction(d, e0.in_direction(d));
      e1.set_direction(d, s0.in_direction(d));
    }
    else
      meep::abort("bug: impossible(?) looping boundaries");
  }
}

// One lattice image of a loop volume (fields::loop_in_chunks,
// src/loop_in_chunks.cpp:355-470, one chunk = the whole cell, no symmetry):
// the owned points of the volume shifted by -shift, their boundary weights,
// and the Bloch phase of the shift.
struct LoopImage {
  LoopBox L;
  ivec shift;
  std::complex<double> phase = 1.0;
};

static LoopBox loop_shifted(const grid_volume &gv, const volume &where, component cgrid, const ivec &is,
                            const ivec &ie, const vec &s0, const vec &s1, const vec &e0, const vec &e1,
                            const ivec &shifti) {
  LoopBox L;
  ivec iscoS = gv.little_owned_corner(cgrid), iecoS = gv.big_owned_corner(cgrid);
  ivec iscS(max(is - shifti, iscoS));
  ivec iecS(min(ie - shifti, iecoS));
  if (!(iscS <= iecS)) return L;
  const ivec isc = iscS, iec = iecS;
  iscS += shifti;
  iecS += shifti;
  vec s0c(gv.dim, 1.0), s1c(gv.dim, 1.0), e0c(gv.dim, 1.0), e1c(gv.dim, 1.0);
  LOOP_OVER_DIRECTIONS(gv.dim, d) {
    if (iscS.in_direction(d) == is.in_direction(d)) {
      s0c.set_direction(d, s0.in_direction(d));
      s1c.set_direction(d, s1.in_direction(d));
    }
    else if (iscS.in_direction(d) == is.in_direction(d) + 2) {
      s0c.set_direction(d, s1.in_direction(d));
    }
    if (iecS.in_direction(d) == ie.in_direction(d)) {
      e0c.set_direction(d, e0.in_direction(d));
      e1c.set_direction(d, e1.in_direction(d));
    }
    else if (iecS.in_direction(d) == ie.in_direction(d) - 2) {
      e0c.set_direction(d, e1.in_direction(d));
    }
    if (iecS.in_direction(d) == iscS.in_direction(d)) {
      double w = std::min(s0c.in_direction(d), e0c.in_direction(d));
      s0c.set_direction(d, w);
      e0c.set_direction(d, w);
      s1c.set_direction(d, w);
      e1c.set_direction(d, w);
    }
    else if (iecS.in_direction(d) == iscS.in_direction(d) + 1 * 2) {
      double w = std::min(s0c.in_direction(d), e1c.in_direction(d));
      s0c.set_direction(d, w);
      e1c.set_direction(d, w);
      w = std::min(s1c.in_direction(d), e0c.in_direction(d));
      s1c.set_direction(d, w);
      e0c.set_direction(d, w);
    }
    else if (iecS.in_direction(d) == iscS.in_direction(d) + 2 * 2) {
      double w = std::min(s1c.in_direction(d), e1c.in_direction(d));
      s1c.set_direction(d, w);
      e1c.set_direction(d, w);
    }
  }
  double dV0 = 1.0;
  LOOP_OVER_DIRECTIONS(gv.dim, d) {
    if (where.in_direction(d) > 0.0) dV0 *= gv.inva;
  }
  L.empty = false;
  L.is = isc;
  L.ie = iec;
  L.s0 = s0c;
  L.s1 = s1c;
  L.e0 = e0c;
  L.e1 = e1c;
  L.dV0 = dV0;
  return L;
}

// every image of `where` along the Bloch-periodic directions (lattice shifts
// from floor((where_min - cell_max) / L) to ceil((where_max - cell_min) / L),
// phase prod eikna^shift); a single unshifted image otherwise
static std::vector<LoopImage> loop_images(const grid_volume &gv, const volume &where, component cgrid,
                                          const int periodic[3], const std::complex<double> eikna[3],
                                          bool snap_empty = false) {
  vec yee_c(gv.yee_shift(Centered) - gv.yee_shift(cgrid));
  ivec iyee_c(gv.iyee_shift(Centered) - gv.iyee_shift(cgrid));
  volume wherec(where + yee_c);
  ivec is(vec2diel_floor(wherec.get_min_corner(), gv.a, zero_ivec(gv.dim)) - iyee_c);
  ivec ie(vec2diel_ceil(wherec.get_max_corner(), gv.a, zero_ivec(gv.dim)) - iyee_c);
  vec s0(gv.dim), e0(gv.dim), s1(gv.dim), e1(gv.dim);
  compute_boundary_weights(gv, where, is, ie, snap_empty, s0, e0, s1, e1);
  const volume gvS = gv.surroundings();
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  LOOP_OVER_DIRECTIONS(gv.dim, d) {
    if (d > Z || !periodic[d]) continue;
    const double L = gv.num_direction(d) * gv.inva;
    lo[d] = int(std::floor((where.in_direction_min(d) - gvS.in_direction_max(d)) / L));
    hi[d] = int(std::ceil((where.in_direction_max(d) - gvS.in_direction_min(d)) / L));
  }
  std::vector<LoopImage> out;
  for (int a = lo[0]; a <= hi[0]; a++)
    for (int b = lo[1]; b <= hi[1]; b++)
      for (int c = lo[2]; c <= hi[2]; c++) {
        const int ish[3] = {a, b, c};
        LoopImage im;
        im.shift = zero_ivec(gv.dim);
        LOOP_OVER_DIRECTIONS(gv.dim, d) {
          if (d > Z) continue;
          im.shift.set_direction(d, 2 * gv.num_direction(d) * ish[d]);
          im.phase *= std::pow(eikna[d], ish[d]);
        }
        im.L = loop_shifted(gv, where, cgrid, is, ie, s0, s1, e0, e1, im.shift);
        if (!im.L.empty) out.push_back(im);
      }
  return out;
}

static LoopBox loop_global(const grid_volume &gv, const volume &where, component cgrid,
                           bool snap_empty = false) {
  const int none[3] = {0, 0, 0};
  const std::complex<double> ones[3] = {1.0, 1.0, 1.0};
  std::vector<LoopImage> im = loop_images(gv, where, cgrid, none, ones, snap_empty);
  return im.empty() ? LoopBox() : im[0].L;
}

// IVEC_LOOP_WEIGHT1x (src/meep/vec.hpp:365-372)
static double w1x(const LoopBox &L, int i, int n, direction d) {
  if (i > 1 && i < n - 2) return 1.0;
  if (i == 0) return L.s0.in_direction(d);
  if (i == 1) return L.s1.in_direction(d);
  if (i == n - 1) return L.e0.in_direction(d);
  if (i == n - 2) return L.e1.in_direction(d);
  return 1.0;
}

/* ------------------------------------------------------ fields: sources */
static std::complex<double> one_amp(const vec &) { return 1.0; }

void fields::add_point_source(component c, double freq, double width, double peaktime,
                              double cutoff, const vec &p, std::complex<double> amp, int is_c) {
  width /= freq;
  if (is_c) {
    continuous_src_time src(freq, width, time(), infinity, cutoff);
    if (is_magnetic(c)) src.is_integrated = false;
    add_point_source(c, src, p, amp);
  }
  else {
    cutoff = gv.inva + cutoff * width;
    if (peaktime <= 0.0) peaktime = time() + cutoff;
    peaktime += is_magnetic(c) ? -dt * 0.5 : dt;
    gaussian_src_time src(freq, width, peaktime - cutoff, peaktime + cutoff);
    if (is_magnetic(c)) src.is_integrated = false;
    add_point_source(c, src, p, amp);
  }
}

void fields::add_point_source(component c, const src_time &src, const vec &p,
                              std::complex<double> amp) {
  add_volume_source(c, src, volume(p, p), amp);
}

void fields::add_volume_source(component c, const src_time &src, const volume &where,
                               std::complex<double> amp) {
  add_volume_source(c, src, where, one_amp, amp);
}

void fields::add_volume_source(component c, const src_time &src, const volume &where_,
                               std::complex<double> A(const vec &), std::complex<double> amp) {
  if (d->sim) meep::abort("sources must be added before the first step in the GB300 engine");
  if (!is_electric(c) && !is_magnetic(c))
    meep::abort("sources on D/B components are not supported by the GB300 engine");
  volume where(where_);
  if (gv.dim != where.dim) meep::abort("incorrect source grid_volume dimensionality in add_volume_source");
  LOOP_OVER_DIRECTIONS(gv.dim, dd) {
    double w = user_volume.boundary_location(High, dd) - user_volume.boundary_location(Low, dd);
    if (where.in_direction(dd) > w + gv.inva)
      meep::abort("Source width > cell width in %s direction!\n", dd == X ? "x" : dd == Y ? "y" : "z");
    else if (where.in_direction(dd) > w) {
      double dw = where.in_direction(dd) - w;
      where.set_direction_min(dd, where.in_direction_min(dd) - dw * 0.5);
      where.set_direction_max(dd, where.in_direction_min(dd) + w);
    }
  }
  std::complex<double> damp = amp;
  LOOP_OVER_DIRECTIONS(gv.dim, dd) {
    if (where.in_direction(dd) == 0.0) damp *= gv.a; // delta-function units
  }
  d->srcs.emplace_back(src.clone());
  int sidx = (int)d->srcs.size() - 1;
  vec center = (where.get_min_corner() + where.get_max_corner()) * 0.5;
  PendingSource ps;
  ps.c = mfd_comp(c);
  ps.src = sidx;
  for (const LoopImage &img : loop_images(gv, where, c, d->periodic, d->eikna)) {
    const LoopBox &L = img.L;
    // src_vol_chunkloop (src/sources.cpp:259-273): amp * conj(shift phase),
    // amplitude function at the unshifted position
    const std::complex<double> iamp = damp * std::conj(img.phase);
    const vec vshift = vec(img.shift.dim, 0.0) + (img.shift * (0.5 * gv.inva));
    Dense dn(gv);
    int k0[3], k1[3], n[3] = {1, 1, 1};
    dn.kof(gv, c, L.is, k0);
    dn.kof(gv, c, L.ie, k1);
    direction ds[3];
    int nd = 0;
    LOOP_OVER_DIRECTIONS(gv.dim, dd) {
      ds[nd] = dd;
      n[nd] = k1[dd] - k0[dd] + 1;
      nd++;
    }
    // loop order / weight product of LOOP_OVER_IVECS and IVEC_LOOP_WEIGHT:
    // loop directions (X,Y,Z) in 3-D, (Z absent, X, Y) in 2-D, (Z) in 1-D
    int k[3];
    int i[3];
    for (i[0] = 0; i[0] < n[0]; i[0]++)
      for (i[1] = 0; i[1] < (nd > 1 ? n[1] : 1); i[1]++)
        for (i[2] = 0; i[2] < (nd > 2 ? n[2] : 1); i[2]++) {
          k[0] = k[1] = k[2] = 0;
          double wd[3] = {1, 1, 1};
          for (int q = 0; q < nd; q++) {
            k[ds[q]] = k0[ds[q]] + i[q];
            wd[q] = w1x(L, i[q], n[q], ds[q]);
          }
          double wgt;
          if (gv.dim == D3) wgt = wd[2] * (wd[1] * (1.0 * wd[0]));
          else if (gv.dim == D2) wgt = wd[1] * (wd[0] * (1.0 * 1.0));
          else wgt = 1.0 * (1.0 * (1.0 * wd[0]));
          ivec iloc = dn.iloc(gv, c, k);
          if (!gv.owns(iloc)) continue;
          vec loc = loop_loc(gv, iloc) + vshift;
          vec rel = loc - center;
          ps.idx.push_back(dn.index(k));
          ps.amp.push_back(wgt * iamp * A(rel));
        }
  }
  d->pending.push_back(std::move(ps));
  d->components = require_components(gv, c, d->components);
}

/* ------------------------------------------------------- fields: DFT */
static int auto_decimation(fields &f, const double *freq, size_t Nfreq) {
  double src_freq_max = 0;
  bool any_cw = false;
  for (const auto &s : f.d->srcs) {
    if (s->get_fwidth() == 0) any_cw = true;
    else src_freq_max = std::max(src_freq_max, std::abs(s->frequency().real()) + 0.5 * s->get_fwidth());
  }
  if (any_cw) return 1;
  double freq_max = 0;
  for (size_t i = 0; i < Nfreq; ++i)
    freq_max = std::max(freq_max, std::abs(freq[i]));
  if ((freq_max > 0) && (src_freq_max > 0))
    return std::max(1, int(std::floor(1 / (f.dt * (freq_max + src_freq_max)))));
  return 1;
}

// fields::add_dft for one component; returns the new chunk (or nullptr if the
// component is not allocated), prepended to `next`.
static dft_chunk *add_dft_one(fields &f, component c, const volume &where, const double *freq,
                              size_t Nfreq, bool include_dV_and_interp_weights,
                              std::complex<double> stored_weight, dft_chunk *next,
                              bool use_centered_grid, int decimation_factor, int vc = -1,
                              bool sqrt_dV_and_interp_weights = false, std::complex<double> extra_weight = 1.0) {
  fields::impl &I = *f.d;
  if (component_direction(c) > Z) return next;
  if (!I.components) meep::abort("allocate field components (by adding sources) before adding dft objects");
  int mc = mfd_comp(c);
  if (!((I.components >> mc) & 1)) return next;
  ensure_engine(f);
  if (decimation_factor == 0) decimation_factor = auto_decimation(f, freq, Nfreq);
  const grid_volume &gv = f.gv;
  component cgrid = use_centered_grid ? Centered : c;
  // one chunk per lattice image of the region (add_dft_chunkloop,
  // src/dft.cpp:158-173: scale times the image's Bloch phase)
  for (const LoopImage &img : loop_images(gv, where, cgrid, I.periodic, I.eikna)) {
  const LoopBox &L = img.L;
  Dense dn(gv);
  // array index box of component c (for the centred grid, point k of c is the
  // base of the average centred at 2k+1)
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  LOOP_OVER_DIRECTIONS(gv.dim, dd) {
    int off = use_centered_grid ? 1 : gv.iyee_shift(c).in_direction(dd);
    lo[dd] = (L.is.in_direction(dd) - gv.little_corner().in_direction(dd) - off) / 2;
    hi[dd] = (L.ie.in_direction(dd) - gv.little_corner().in_direction(dd) - off) / 2;
  }
  std::vector<double> w[3];
  const double *wp[3] = {nullptr, nullptr, nullptr};
  LOOP_OVER_DIRECTIONS(gv.dim, dd) {
    int n = hi[dd] - lo[dd] + 1;
    w[dd].resize(n);
    for (int i = 0; i < n; i++)
      w[dd][i] = w1x(L, i, n, dd);
    wp[dd] = w[dd].data();
  }
  std::complex<double> scale = stored_weight * img.phase *
                               (f.dt / std::sqrt(2.0 * pi) * decimation_factor);
  int id = -1;
  const int incl = include_dV_and_interp_weights ? (sqrt_dV_and_interp_weights ? 2 : 1) : 0;
  chk(mfd_add_dft(I.sim, mc, lo, hi, wp, L.dV0, incl, scale.real(),
                  scale.imag(), use_centered_grid ? 1 : 0, Nfreq, freq, decimation_factor, &id));
  std::unique_ptr<dft_chunk> ch(new dft_chunk);
  ch->c = c;
  ch->vc = vc < 0 ? int(c) : vc;
  ch->extra_weight = extra_weight;
  ch->monitor_id = id;
  ch->decimation_factor = decimation_factor;
  ch->fld = &f;
  ch->is = L.is;
  ch->ie = L.ie;
  ch->shift = img.shift;
  ch->omega.resize(Nfreq);
  for (size_t i = 0; i < Nfreq; i++)
    ch->omega[i] = 2 * pi * freq[i];
  size_t npts = 1;
  LOOP_OVER_DIRECTIONS(gv.dim, dd) npts *= (size_t)(hi[dd] - lo[dd] + 1);
  ch->N = npts;
  ch->dft = new std::complex<realnum>[npts * Nfreq]();
  ch->next_in_dft = next;
  next = ch.get();
  I.chunks.push_back(std::move(ch));
  }
  return next;
}

dft_flux fields::add_dft_flux(const volume_list *where_, const double *freq, size_t Nfreq,
                              bool use_symmetry, bool centered_grid, int decimation_factor) {
  (void)use_symmetry;
  dft_flux fl;
  fl.f = this;
  fl.freq.assign(freq, freq + Nfreq);
  if (!where_) return fl;
  dft_chunk *E = nullptr, *H = nullptr;
  component cE[2] = {Ex, Ey}, cH[2] = {Hy, Hx};
  for (const volume_list *where = where_; where; where = where->next) {
    switch (where->c) {
      case Sx: cE[0] = Ey, cE[1] = Ez, cH[0] = Hz, cH[1] = Hy; break;
      case Sy: cE[0] = Ez, cE[1] = Ex, cH[0] = Hx, cH[1] = Hz; break;
      case Sz: cE[0] = Ex, cE[1] = Ey, cH[0] = Hy, cH[1] = Hx; break;
      default: meep::abort("invalid flux component!");
    }
    for (int i = 0; i < 2; ++i) {
      E = add_dft_one(*this, cE[i], where->v, freq, Nfreq, true, where->weight * double(1 - 2 * i), E,
                      centered_grid, decimation_factor);
      H = add_dft_one(*this, cH[i], where->v, freq, Nfreq, false, 1.0, H, centered_grid,
                      decimation_factor);
    }
  }
  fl.E = E;
  fl.H = H;
  fl.cE = cE[0];
  fl.cH = cH[0];
  return fl;
}

dft_flux fields::add_dft_flux(direction dd, const volume &where, double freq_min, double freq_max,
                              int Nfreq, bool use_symmetry, bool centered_grid, int decimation_factor) {
  return add_dft_flux(dd, where, linspace(freq_min, freq_max, Nfreq), use_symmetry, centered_grid,
                      decimation_factor);
}

dft_flux fields::add_dft_flux(direction dd, const volume &where, const std::vector<double> &freq,
                              bool use_symmetry, bool centered_grid, int decimation_factor) {
  volume_list vl(where, direction_component(Sx, dd));
  return add_dft_flux(&vl, freq.data(), freq.size(), use_symmetry, centered_grid, decimation_factor);
}

dft_flux fields::add_dft_flux_plane(const volume &where, double freq_min, double freq_max,
                                    int Nfreq) {
  direction dd = NO_DIRECTION;
  LOOP_OVER_DIRECTIONS(gv.dim, q) {
    if (where.in_direction(q) == 0) dd = q;
  }
  if (dd == NO_DIRECTION) meep::abort("add_dft_flux_plane needs a plane");
  return add_dft_flux(dd, where, freq_min, freq_max, Nfreq);
}

dft_fields fields::add_dft_fields(component *components, int num_components, const volume where,
                                  const double *freq, size_t Nfreq, bool use_centered_grid,
                                  int decimation_factor, bool persist) {
  if (persist) meep::abort("persistent DFT fields are not supported by the GB300 engine");
  dft_chunk *chunks = nullptr;
  for (int nc = 0; nc < num_components; nc++)
    chunks = add_dft_one(*this, components[nc], where, freq, Nfreq, false, 1.0, chunks,
                         use_centered_grid, decimation_factor);
  return dft_fields(chunks, std::vector<double>(freq, freq + Nfreq), where);
}

dft_fields fields::add_dft_fields(component *components, int num_components, const volume where,
                                  double freq_min, double freq_max, int Nfreq,
                                  bool use_centered_grid, int decimation_factor, bool persist) {
  std::vector<double> fr = linspace(freq_min, freq_max, Nfreq);
  return add_dft_fields(components, num_components, where, fr.data(), fr.size(),
                        use_centered_grid, decimation_factor, persist);
}

double *dft_flux::flux() {
  size_t nf = freq.size();
  double *F = new double[nf];
  for (size_t i = 0; i < nf; i++)
    F[i] = 0;
  std::vector<int> idE, idH;
  for (dft_chunk *e = E, *h = H; e && h; e = e->next_in_dft, h = h->next_in_dft) {
    idE.push_back(e->monitor_id);
    idH.push_back(h->monitor_id);
  }
  if (!idE.empty()) chk(mfd_flux(f->d->sim, (int)idE.size(), idE.data(), idH.data(), F));
  return F;
}

void fields::sync_dfts() {
  if (!d->sim) return;
  for (auto &ch : d->chunks) {
    size_t np = 0, nf = 0;
    chk(mfd_get_dft(d->sim, ch->monitor_id, nullptr, &np, &nf));
    std::vector<double> buf(2 * np * nf);
    chk(mfd_get_dft(d->sim, ch->monitor_id, buf.data(), &np, &nf));
    for (size_t i = 0; i < np * nf; i++)
      ch->dft[i] = std::complex<realnum>(realnum(buf[2 * i]), realnum(buf[2 * i + 1]));
  }
}

void sync_dfts(fields &f) { f.sync_dfts(); }

double fields::last_source_time() const {
  double t = 0;
  for (const auto &src : d->srcs)
    t = std::max(t, src->last_time());
  return t;
}

/* ------------------------------------------------------- fields: step */
void fields::step() {
  ensure_engine(*this);
  chk(mfd_step(d->sim, 1));
  t += 1;
}

void step_n(fields &f, int n) {
  ensure_engine(f);
  chk(mfd_step(f.d->sim, n));
  f.t += n;
}

double fields::last_step_ms() const { return d->sim ? mfd_last_step_ms(d->sim) : 0.0; }
long long fields::kernel_launches() const { return d->sim ? mfd_kernel_launches(d->sim) : 0; }

std::vector<double> fields::get_field_array(component c) {
  ensure_engine(*this);
  Dense dn(gv);
  std::vector<double> out(dn.count(), 0.0);
  int mc = mfd_comp(c);
  chk(mfd_get_field(d->sim, mc, out.data()));
  return out;
}

std::complex<double> fields::get_field(component c, const ivec &iloc_, bool parallel) {
  (void)parallel;
  if (c >= Dielectric) meep::abort("get_field of a non-field component is not supported");
  ivec iloc = iloc_;
  std::complex<double> phase = 1.0;
  // points outside the cell along a periodic direction are translated into it
  // with the Bloch phase (fields::locate_point_in_user_volume,
  // src/boundaries.cpp:207-229)
  if (!gv.owns(iloc))
    LOOP_OVER_DIRECTIONS(gv.dim, dd) {
      if (dd > Z || !d->periodic[dd]) continue;
      const int L = 2 * gv.num_direction(dd), lo = gv.little_corner().in_direction(dd);
      while (iloc.in_direction(dd) <= lo) {
        iloc.set_direction(dd, iloc.in_direction(dd) + L);
        phase *= std::conj(d->eikna[dd]);
      }
      while (iloc.in_direction(dd) - L > lo) {
        iloc.set_direction(dd, iloc.in_direction(dd) - L);
        phase *= d->eikna[dd];
      }
    }
  if (!gv.owns(iloc)) return 0.0;
  int mc = mfd_comp(c);
  if (!((d->components >> mc) & 1)) return 0.0;
  ensure_engine(*this);
  if (d->cache_t[mc] != t) {
    d->cache[mc] = get_field_array(c);
    if (d->complex_fields()) {
      d->cache_im[mc].assign(d->cache[mc].size(), 0.0);
      chk(mfd_get_field_im(d->sim, mc, d->cache_im[mc].data()));
    }
    d->cache_t[mc] = t;
  }
  Dense dn(gv);
  int k[3];
  dn.kof(gv, c, iloc, k);
  // points not on this component's grid are not owned by it
  ivec back = dn.iloc(gv, c, k);
  if (back != iloc) return 0.0;
  const double im = d->complex_fields() ? d->cache_im[mc][dn.index(k)] : 0.0;
  return phase * std::complex<double>(d->cache[mc][dn.index(k)], im);
}

static int my_round(double x) { return int(std::floor(std::fabs(x) + 0.5) * (x < 0 ? -1 : 1)); }

static void stupidsort(ivec *locs, double *w, int l) {
  while (l) {
    if (std::fabs(w[0]) < 2e-15) {
      w[0] = w[l - 1];
      locs[0] = locs[l - 1];
      w[l - 1] = 0.0;
      locs[l - 1] = ivec(locs[0].dim, 0);
    }
    else {
      w += 1;
      locs += 1;
    }
    l -= 1;
  }
}

// grid_volume::interpolate(component, vec, ivec[8], double[8]) (src/vec.cpp:555-612)
static void interpolate(const grid_volume &gv, component c, const vec &pc, ivec locs[8],
                        double weights[8]) {
  const double SMALL = 1e-13;
  const vec p = (pc - gv.yee_shift(c)) * gv.a;
  ivec middle(gv.dim);
  LOOP_OVER_DIRECTIONS(gv.dim, dd) middle.set_direction(dd, ((int)std::floor(p.in_direction(dd))) * 2 + 1);
  middle += gv.iyee_shift(c);
  const vec midv = gv[middle];
  const vec dv = (pc - midv) * (2 * gv.a);
  int already_have = 1;
  ivec rv(gv.dim);
  LOOP_OVER_DIRECTIONS(gv.dim, dd) rv.set_direction(dd, my_round(midv.in_direction(dd) * 2 * gv.a));
  for (int i = 0; i < 8; i++) {
    locs[i] = rv;
    weights[i] = 1.0;
  }
  LOOP_OVER_DIRECTIONS(gv.dim, dd) {
    for (int i = 0; i < already_have; i++) {
      locs[already_have + i] = locs[i];
      weights[already_have + i] = weights[i];
      locs[i].set_direction(dd, middle.in_direction(dd) - 1);
      weights[i] *= 0.5 * (1.0 - dv.in_direction(dd));
      locs[already_have + i].set_direction(dd, middle.in_direction(dd) + 1);
      weights[already_have + i] *= 0.5 * (1.0 + dv.in_direction(dd));
    }
    already_have *= 2;
  }
  for (int i = already_have; i < 8; i++)
    weights[i] = 0.0;
  double total_weight = 0.0;
  for (int i = 0; i < already_have; i++)
    total_weight += weights[i];
  for (int i = 0; i < already_have; i++)
    weights[i] += (1.0 - total_weight) * (1.0 / already_have);
  for (int i = 0; i < already_have; i++) {
    if (weights[i] < 0.0) {
      if (-weights[i] >= SMALL * 1e5) meep::abort("large negative interpolation weight");
      weights[i] = 0.0;
    }
    else if (weights[i] < SMALL)
      weights[i] = 0.0;
  }
  stupidsort(locs, weights, already_have);
  bool all_same = true;
  for (int i = 0; i < 8 && weights[i]; i++)
    if (weights[i] != weights[0]) all_same = false;
  if (all_same) {
    int num_weights = 0;
    for (int i = 0; i < 8 && weights[i]; i++)
      num_weights++;
    for (int i = 0; i < 8 && weights[i]; i++)
      weights[i] = 1.0 / num_weights;
  }
}

std::complex<double> fields::get_field(component c, const vec &loc, bool parallel) {
  (void)parallel;
  ivec ilocs[8];
  double w[8];
  std::complex<double> res = 0.0;
  interpolate(gv, c, loc, ilocs, w);
  for (int argh = 0; argh < 8 && w[argh]; argh++)
    res += w[argh] * get_field(c, ilocs[argh], false);
  return res;
}

/* ------------------------------------------------------- near-to-far */
volume volume::operator|(const volume &a) const {
  vec lo(dim), hi(dim);
  LOOP_OVER_DIRECTIONS(dim, dd) {
    lo.set_direction(dd, std::min(in_direction_min(dd), a.in_direction_min(dd)));
    hi.set_direction(dd, std::max(in_direction_max(dd), a.in_direction_max(dd)));
  }
  return volume(lo, hi);
}

// volume::normal_direction (src/vec.cpp:227-262): the one empty direction
static direction normal_direction(const volume &v) {
  direction d = NO_DIRECTION;
  switch (v.dim) {
    case D1: d = Z; break;
    case D2:
      if (v.in_direction(X) == 0 && v.in_direction(Y) > 0) d = X;
      else if (v.in_direction(X) > 0 && v.in_direction(Y) == 0) d = Y;
      break;
    case D3: {
      const bool zx = v.in_direction(X) == 0, zy = v.in_direction(Y) == 0, zz = v.in_direction(Z) == 0;
      if (zx && !zy && !zz) d = X;
      else if (!zx && zy && !zz) d = Y;
      else if (!zx && !zy && zz) d = Z;
      break;
    }
    default: break;
  }
  return d;
}

void dft_chunk::scale_dft(std::complex<double> scale) {
  for (dft_chunk *ch = this; ch; ch = ch->next_in_dft) {
    if (ch->fld && ch->fld->d->sim) chk(mfd_scale_dft(ch->fld->d->sim, ch->monitor_id, scale.real(), scale.imag()));
    for (size_t i = 0; i < ch->N * ch->omega.size(); ++i)
      ch->dft[i] *= scale;
  }
}

// fields::get_chi1inv(c, d, ivec) (src/monitor.cpp:135-154): vacuum outside
// the cell
static std::complex<double> field_chi1inv(const fields &f, component c, direction dd, const ivec &iloc) {
  if (!f.gv.owns(iloc)) return dd == component_direction(c) ? 1.0 : 0.0;
  return f.s->get_chi1inv(c, dd, iloc);
}

// fields::get_eps / get_mu (src/monitor.cpp:172-194): n / sum over the
// grid's E (H) components of the interpolated diagonal chi1inv
static std::complex<double> trace_average(const fields &f, bool electric, const vec &loc) {
  std::complex<double> tr(0.0, 0.0);
  int nc = 0;
  const component cs[3] = {electric ? Ex : Hx, electric ? Ey : Hy, electric ? Ez : Hz};
  for (component c : cs) {
    if (!f.gv.has_field(c)) continue;
    ivec ilocs[8];
    double w[8];
    std::complex<double> res(0.0, 0.0);
    interpolate(f.gv, c, loc, ilocs, w);
    for (int k = 0; k < 8 && w[k] != 0; k++)
      res += w[k] * field_chi1inv(f, c, component_direction(c), ilocs[k]);
    tr += res;
    ++nc;
  }
  return std::complex<double>(nc, 0) / tr;
}

std::complex<double> fields::get_eps(const vec &loc, double frequency) const {
  if (frequency != 0) meep::abort("frequency-dependent eps is not supported by the GB300 engine");
  return trace_average(*this, true, loc);
}

std::complex<double> fields::get_mu(const vec &loc, double frequency) const {
  if (frequency != 0) meep::abort("frequency-dependent mu is not supported by the GB300 engine");
  return trace_average(*this, false, loc);
}

static bool approxeq(double a, double b) { return std::fabs(a - b) < 0.5e-11 * (std::fabs(a) + std::fabs(b)); }

// fields::add_dft_near2far (src/near2far.cpp:569-651): per surface, the two
// tangential E and H components as DFT chunks on their own Yee grids, each
// standing for the equivalent current n x H (electric) or -n x E (magnetic)
// of the perpendicular tangential component, with the sign of n x c
dft_near2far fields::add_dft_near2far(const volume_list *where, const double *freq, size_t Nfreq,
                                      int decimation_factor, int Nperiods) {
  dft_chunk *F = nullptr;
  double eps = 0, mu = 0;
  volume everywhere = where->v;
  direction periodic_d[2] = {NO_DIRECTION, NO_DIRECTION};
  int periodic_n[2] = {0, 0};
  double periodic_k[2] = {0, 0}, period[2] = {0, 0};
  for (const volume_list *w = where; w; w = w->next) {
    everywhere = everywhere | where->v; // (the reference unions the first surface with itself)
    direction nd = w->c >= Sx ? component_direction(derived_component(w->c)) : component_direction(component(w->c));
    if (nd == NO_DIRECTION) nd = normal_direction(w->v);
    if (nd == NO_DIRECTION) meep::abort("unknown dft_near2far normal");
    const double weps = get_eps(w->v.center()).real();
    const double wmu = get_mu(w->v.center()).real();
    if (w != where && !(approxeq(eps, weps) && approxeq(mu, wmu)))
      meep::abort("dft_near2far requires surfaces in a homogeneous medium");
    eps = weps;
    mu = wmu;
    // transverse directions in cyclic order (sign s below)
    direction fd[2];
    switch (nd) {
      case X: fd[0] = Y, fd[1] = Z; break;
      case Y: fd[0] = Z, fd[1] = X; break;
      case Z: fd[0] = X, fd[1] = Y; break;
      default: meep::abort("invalid normal direction in dft_near2far!");
    }
    if (Nperiods > 1) {
      for (int i = 0; i < 2; ++i) {
        const double user_width = user_volume.num_direction(fd[i]) / a;
        const bool has = gv.dim == D3 || (gv.dim == D2 && fd[i] != Z);
        if (has && d->periodic[fd[i]] && float(w->v.in_direction(fd[i])) >= float(user_width)) {
          periodic_d[i] = fd[i];
          periodic_n[i] = Nperiods;
          period[i] = user_width;
          periodic_k[i] = 2 * pi * d->kvec[fd[i]] * period[i];
        }
      }
    }
    for (int i = 0; i < 2; ++i) {   // E or H
      for (int j = 0; j < 2; ++j) { // first or second transverse component
        const component c = direction_component(i == 0 ? Ex : Hx, fd[j]);
        const component c0 = direction_component(i == 0 ? Hx : Ex, fd[1 - j]);
        double sgn = j == 0 ? 1 : -1;
        if (is_electric(c)) sgn = -sgn;
        F = add_dft_one(*this, c, w->v, freq, Nfreq, true, sgn * w->weight, F, false, decimation_factor, int(c0));
      }
    }
  }
  return dft_near2far(F, freq, Nfreq, eps, mu, everywhere, periodic_d, periodic_n, periodic_k, period);
}

dft_near2far fields::add_dft_near2far(const volume_list *where, double freq_min, double freq_max, int Nfreq,
                                      int decimation_factor, int Nperiods) {
  std::vector<double> fr = linspace(freq_min, freq_max, Nfreq);
  return add_dft_near2far(where, fr.data(), fr.size(), decimation_factor, Nperiods);
}

dft_near2far fields::add_dft_near2far(const volume_list *where, const std::vector<double> &freq,
                                      int decimation_factor, int Nperiods) {
  return add_dft_near2far(where, freq.data(), freq.size(), decimation_factor, Nperiods);
}

dft_near2far::dft_near2far(dft_chunk *F_, const double *freq_, size_t Nfreq, double eps_, double mu_,
                           const volume &where_, const direction periodic_d_[2], const int periodic_n_[2],
                           const double periodic_k_[2], const double period_[2])
    : freq(freq_, freq_ + Nfreq), F(F_), eps(eps_), mu(mu_), where(where_) {
  for (int i = 0; i < 2; ++i) {
    periodic_d[i] = periodic_d_[i];
    periodic_n[i] = periodic_n_[i];
    periodic_k[i] = periodic_k_[i];
    period[i] = period_[i];
  }
}

void dft_near2far::scale_dfts(std::complex<double> scale) {
  if (F) F->scale_dft(scale);
}

void dft_near2far::remove() {
  // the chunks stay owned by their fields (and their device sums allocated);
  // the list is only detached
  F = nullptr;
}

void dft_near2far::farfields_at(const std::vector<vec> &pts, std::complex<double> *out) {
  const size_t Nfreq = freq.size();
  if (pts.empty() || Nfreq == 0) return;
  if (!F) {
    for (size_t i = 0; i < pts.size() * 6 * Nfreq; i++)
      out[i] = 0.0;
    return;
  }
  fields &f = *F->fld;
  std::vector<int> ids, c0;
  std::vector<double> is_half, rshift;
  for (dft_chunk *ch = F; ch; ch = ch->next_in_dft) {
    ids.push_back(ch->monitor_id);
    c0.push_back(mfd_comp(component(ch->vc)));
    if (ch->omega.size() != Nfreq) meep::abort("near2far chunk with a different number of frequencies");
    const vec rs = ch->shift * (0.5 * f.gv.inva);
    for (int q = 0; q < 3; q++) {
      const direction dd = direction(q);
      const bool has = f.gv.dim == D3 || (f.gv.dim == D2 && dd != Z);
      is_half.push_back(has ? 0.5 * ch->is.in_direction(dd) : 0.0);
      rshift.push_back(has ? rs.in_direction(dd) : 0.0);
    }
  }
  std::vector<double> xs(3 * pts.size());
  for (size_t k = 0; k < pts.size(); k++) {
    if (pts[k].dim != f.gv.dim) meep::abort("far-field point dimensions differ from the grid's");
    xs[3 * k] = pts[k].x();
    xs[3 * k + 1] = pts[k].y();
    xs[3 * k + 2] = pts[k].dim == D3 ? pts[k].z() : 0.0;
  }
  int pd[2], pn[2];
  for (int i = 0; i < 2; i++) {
    pd[i] = periodic_d[i] == NO_DIRECTION ? -1 : int(periodic_d[i]);
    pn[i] = periodic_d[i] == NO_DIRECTION ? 0 : periodic_n[i];
  }
  chk(mfd_farfield(f.d->sim, (int)ids.size(), ids.data(), c0.data(), is_half.data(), rshift.data(), eps, mu, pd, pn,
                   periodic_k, period, (int64_t)pts.size(), xs.data(), reinterpret_cast<double *>(out)));
}

void dft_near2far::farfield_lowlevel(std::complex<double> *EH, const vec &x, double greencyl_tol) {
  (void)greencyl_tol;
  if (x.dim != D3 && x.dim != D2) meep::abort("only 2d or 3d far-field computation is supported");
  farfields_at(std::vector<vec>(1, x), EH);
}

std::complex<double> *dft_near2far::farfield(const vec &x, double greencyl_tol) {
  std::complex<double> *EH = new std::complex<double>[6 * freq.size()];
  farfield_lowlevel(EH, x, greencyl_tol);
  return EH;
}

// dft_near2far::get_farfields_array (src/near2far.cpp:392-467): the grid of
// far points over `where`, all evaluated in one engine call
double *dft_near2far::get_farfields_array(const volume &where, int &rank, size_t *dims, size_t &N, double resolution,
                                          double greencyl_tol) {
  (void)greencyl_tol;
  double dx[3] = {0, 0, 0};
  direction dirs[3] = {X, Y, Z};
  rank = 0;
  N = dims[0] = dims[1] = dims[2] = 1;
  LOOP_OVER_DIRECTIONS(where.dim, dd) {
    dims[rank] = int(std::floor(where.in_direction(dd) * resolution));
    if (dims[rank] <= 1) dims[rank] = 1;
    else dx[rank] = where.in_direction(dd) / (dims[rank] - 1);
    N *= dims[rank];
    dirs[rank++] = dd;
  }
  const size_t Nfreq = freq.size();
  if (N * Nfreq < 1) return NULL;
  std::vector<vec> pts;
  pts.reserve(N);
  vec x(where.dim);
  for (size_t i0 = 0; i0 < dims[0]; ++i0) {
    x.set_direction(dirs[0], where.in_direction_min(dirs[0]) + i0 * dx[0]);
    for (size_t i1 = 0; i1 < dims[1]; ++i1) {
      x.set_direction(dirs[1], where.in_direction_min(dirs[1]) + i1 * dx[1]);
      for (size_t i2 = 0; i2 < dims[2]; ++i2) {
        x.set_direction(dirs[2], where.in_direction_min(dirs[2]) + i2 * dx[2]);
        pts.push_back(x);
      }
    }
  }
  std::vector<std::complex<double>> EH1(pts.size() * 6 * Nfreq);
  farfields_at(pts, EH1.data());
  double *EH = new double[6 * 2 * N * Nfreq];
  for (size_t idx = 0; idx < N; ++idx)
    for (size_t i = 0; i < Nfreq; ++i)
      for (int k = 0; k < 6; ++k) {
        EH[((k * 2 + 0) * N + idx) * Nfreq + i] = EH1[(idx * Nfreq + i) * 6 + k].real();
        EH[((k * 2 + 1) * N + idx) * Nfreq + i] = EH1[(idx * Nfreq + i) * 6 + k].imag();
      }
  int ireduced = 0;
  for (int i = 0; i < rank; ++i)
    if (dims[i] > 1) dims[ireduced++] = dims[i];
  rank = ireduced;
  return EH;
}

// dft_near2far::flux (src/near2far.cpp:517-567): Re(E x H*) . n summed over
// the far-field grid times its area element
double *dft_near2far::flux(direction df, const volume &where, double resolution) {
  if (df > Z || (where.dim == D2 && df == Z) || (where.dim == D1 && df != Z))
    meep::abort("cannot get flux for near2far: co-ordinate mismatch");
  size_t dims[4] = {1, 1, 1, 1};
  int rank = 0;
  size_t N = 1;
  double *EH = get_farfields_array(where, rank, dims, N, resolution);
  const size_t Nfreq = freq.size();
  double *F = new double[Nfreq];
  for (size_t i = 0; i < Nfreq; ++i)
    F[i] = 0;
  std::complex<double> ff[6], cE[2], cH[2];
  for (size_t idx = 0; idx < N; ++idx) {
    for (size_t i = 0; i < Nfreq; ++i) {
      for (int k = 0; k < 6; ++k)
        ff[k] = std::complex<double>(EH[((k * 2 + 0) * N + idx) * Nfreq + i], EH[((k * 2 + 1) * N + idx) * Nfreq + i]);
      switch (df) {
        case X: cE[0] = ff[1], cE[1] = ff[2], cH[0] = ff[5], cH[1] = ff[4]; break;
        case Y: cE[0] = ff[2], cE[1] = ff[0], cH[0] = ff[3], cH[1] = ff[5]; break;
        default: cE[0] = ff[0], cE[1] = ff[1], cH[0] = ff[4], cH[1] = ff[3]; break;
      }
      for (int j = 0; j < 2; ++j)
        F[i] += real(cE[j] * conj(cH[j])) * (1 - 2 * j);
    }
  }
  double dV = 1;
  LOOP_OVER_DIRECTIONS(where.dim, dd) {
    const int n = int(std::floor(where.in_direction(dd) * resolution));
    if (n > 1) dV *= where.in_direction(dd) / (n - 1);
  }
  for (size_t i = 0; i < Nfreq; ++i)
    F[i] *= dV;
  delete[] EH;
  return F;
}

static void green_call(int dim, std::complex<double> *EH, const vec &x, double freq, double eps, double mu,
                       const vec &x0, component c0, std::complex<double> f0) {
  const double xa[3] = {x.x(), x.y(), dim == 3 ? x.z() : 0.0};
  const double xb[3] = {x0.x(), x0.y(), dim == 3 ? x0.z() : 0.0};
  if (!is_electric(c0) && !is_magnetic(c0)) meep::abort("unrecognized source type");
  chk(mfd_green(dim, mfd_comp(c0), freq, eps, mu, f0.real(), f0.imag(), 1, xa, xb, reinterpret_cast<double *>(EH)));
}

void green3d(std::complex<double> *EH, const vec &x, double freq, double eps, double mu, const vec &x0,
             component c0, std::complex<double> f0) {
  if (x.dim != D3) meep::abort("wrong dimensionality in green3d");
  green_call(3, EH, x, freq, eps, mu, x0, c0, f0);
}

void green2d(std::complex<double> *EH, const vec &x, double freq, double eps, double mu, const vec &x0,
             component c0, std::complex<double> f0) {
  if (x.dim != D2) meep::abort("wrong dimensionality in green2d");
  green_call(2, EH, x, freq, eps, mu, x0, c0, f0);
}

/* -------------------------------------------------------- stress / force */
// fields::add_dft_force (src/stress.cpp:139-196): on a surface with normal n,
// the force along f is the Maxwell stress integral.  f != n: E_f E_n* +
// H_f H_n* (offdiag1 with dV weights and the surface weight, offdiag2
// without); f == n: (+1/2 along f, -1/2 across) |E_d|^2 + |H_d|^2 over every
// field direction d, each chunk with the square root of its dV weight and
// the +-1/2 as its extra weight.
dft_force fields::add_dft_force(const volume_list *where, const double *freq, size_t Nfreq, int decimation_factor) {
  dft_chunk *offdiag1 = nullptr, *offdiag2 = nullptr, *diag = nullptr;
  if (!where) return dft_force(offdiag1, offdiag2, diag, freq, Nfreq, volume(gv.center()));
  volume everywhere = where->v;
  for (const volume_list *w = where; w; w = w->next) {
    const direction nd = normal_direction(w->v);
    if (nd == NO_DIRECTION) meep::abort("cannot determine dft_force normal");
    const direction fd = w->c >= Sx ? component_direction(derived_component(w->c)) : component_direction(component(w->c));
    if (fd == NO_DIRECTION) meep::abort("NO_DIRECTION dft_force is invalid");
    if (fd > Z) meep::abort("coordinate-type mismatch in add_dft_force");
    if (fd != nd) {
      offdiag1 = add_dft_one(*this, direction_component(Ex, fd), w->v, freq, Nfreq, true, w->weight, offdiag1, true,
                             decimation_factor);
      offdiag2 = add_dft_one(*this, direction_component(Ex, nd), w->v, freq, Nfreq, false, 1.0, offdiag2, true,
                             decimation_factor);
      offdiag1 = add_dft_one(*this, direction_component(Hx, fd), w->v, freq, Nfreq, true, w->weight, offdiag1, true,
                             decimation_factor);
      offdiag2 = add_dft_one(*this, direction_component(Hx, nd), w->v, freq, Nfreq, false, 1.0, offdiag2, true,
                             decimation_factor);
    }
    else
      for (int q = X; q <= Z; q++) {
        const direction d = direction(q);
        const std::complex<double> weight1 = w->weight * (d == fd ? +0.5 : -0.5);
        diag = add_dft_one(*this, direction_component(Ex, d), w->v, freq, Nfreq, true, 1.0, diag, false,
                           decimation_factor, -1, true, weight1);
        diag = add_dft_one(*this, direction_component(Hx, d), w->v, freq, Nfreq, true, 1.0, diag, false,
                           decimation_factor, -1, true, weight1);
      }
    everywhere = everywhere | w->v;
  }
  return dft_force(offdiag1, offdiag2, diag, freq, Nfreq, everywhere);
}

dft_force fields::add_dft_force(const volume_list *where, double freq_min, double freq_max, int Nfreq,
                                int decimation_factor) {
  std::vector<double> fr = linspace(freq_min, freq_max, Nfreq);
  return add_dft_force(where, fr.data(), fr.size(), decimation_factor);
}

dft_force fields::add_dft_force(const volume_list *where, const std::vector<double> &freq, int decimation_factor) {
  return add_dft_force(where, freq.data(), freq.size(), decimation_factor);
}

dft_force::dft_force(dft_chunk *offdiag1_, dft_chunk *offdiag2_, dft_chunk *diag_, const double *freq_, size_t Nfreq,
                     const volume &where_)
    : freq(freq_, freq_ + Nfreq), offdiag1(offdiag1_), offdiag2(offdiag2_), diag(diag_), where(where_) {}

// dft_force::force (src/stress.cpp:84-96): sum over chunk pairs of
// Re(extra_weight F1 conj(F2)); each pair reduced on the GPU (mfd_flux)
double *dft_force::force() {
  const size_t nf = freq.size();
  double *F = new double[nf];
  for (size_t i = 0; i < nf; i++)
    F[i] = 0;
  std::vector<double> part(nf);
  auto pairs = [&](dft_chunk *a, dft_chunk *b) {
    for (; a && b; a = a->next_in_dft, b = b->next_in_dft) {
      const int ia = a->monitor_id, ib = b->monitor_id;
      chk(mfd_flux(a->fld->d->sim, 1, &ia, &ib, part.data()));
      // Re(w z) with z = sum F1 conj(F2) real for the diagonal (F1 = F2) and
      // w = 1 off the diagonal
      for (size_t i = 0; i < nf; i++)
        F[i] += a->extra_weight.real() * part[i];
    }
  };
  pairs(offdiag1, offdiag2);
  pairs(diag, diag);
  return F;
}

void dft_force::scale_dfts(std::complex<double> scale) {
  if (offdiag1) offdiag1->scale_dft(scale);
  if (offdiag2) offdiag2->scale_dft(scale);
  if (diag) diag->scale_dft(scale);
}

/* ------------------------------------------------- DFT data save / load */
void dft_flux::scale_dfts(std::complex<double> scale) {
  if (E) E->scale_dft(scale);
  if (H) H->scale_dft(scale);
}

size_t dft_data_size(dft_chunk *chunks) {
  size_t n = 0;
  for (dft_chunk *c = chunks; c; c = c->next_in_dft)
    n += c->N * c->omega.size();
  return n;
}

// _get_dft_data / _load_dft_data (python/meep.i:492-527): the chunks' sums
// in list order
void get_dft_data(dft_chunk *chunks, std::complex<double> *data, size_t n) {
  if (n != dft_data_size(chunks))
    meep::abort("Total dft_chunks size does not agree with size allocated for output array.\n");
  size_t at = 0;
  for (dft_chunk *c = chunks; c; c = c->next_in_dft) {
    size_t np = 0, nf = 0;
    chk(mfd_get_dft(c->fld->d->sim, c->monitor_id, reinterpret_cast<double *>(data + at), &np, &nf));
    at += np * nf;
  }
}

void load_dft_data(dft_chunk *chunks, const std::complex<double> *data, size_t n) {
  if (n != dft_data_size(chunks))
    meep::abort("Total dft_chunks size does not agree with size allocated for output array.\n");
  size_t at = 0;
  for (dft_chunk *c = chunks; c; c = c->next_in_dft) {
    const size_t m = c->N * c->omega.size();
    chk(mfd_set_dft(c->fld->d->sim, c->monitor_id, reinterpret_cast<const double *>(data + at)));
    for (size_t i = 0; i < m; i++)
      c->dft[i] = std::complex<realnum>(realnum(data[at + i].real()), realnum(data[at + i].imag()));
    at += m;
  }
}

/* ---------------------------------------------------------------- energy */
// fields::add_dft_energy (src/dft.cpp:725-750): E, D, H, B of every field
// direction on the centred grid, the dV weights on E and H
dft_energy fields::add_dft_energy(const volume_list *where, const double *freq, size_t Nfreq, int decimation_factor) {
  dft_chunk *E = nullptr, *D = nullptr, *H = nullptr, *B = nullptr;
  if (!where) return dft_energy(E, H, D, B, freq, Nfreq, volume(gv.center()));
  const volume firstvol(where->v);
  for (const volume_list *w = where; w; w = w->next)
    for (int q = X; q <= Z; q++) {
      const direction d = direction(q);
      E = add_dft_one(*this, direction_component(Ex, d), w->v, freq, Nfreq, true, 1.0, E, true, decimation_factor);
      D = add_dft_one(*this, direction_component(Dx, d), w->v, freq, Nfreq, false, 1.0, D, true, decimation_factor);
      H = add_dft_one(*this, direction_component(Hx, d), w->v, freq, Nfreq, true, 1.0, H, true, decimation_factor);
      B = add_dft_one(*this, direction_component(Bx, d), w->v, freq, Nfreq, false, 1.0, B, true, decimation_factor);
    }
  return dft_energy(E, H, D, B, freq, Nfreq, firstvol);
}

dft_energy fields::add_dft_energy(const volume_list *where, double freq_min, double freq_max, int Nfreq,
                                  int decimation_factor) {
  std::vector<double> fr = linspace(freq_min, freq_max, Nfreq);
  return add_dft_energy(where, fr.data(), fr.size(), decimation_factor);
}

dft_energy fields::add_dft_energy(const volume_list *where, const std::vector<double> &freq, int decimation_factor) {
  return add_dft_energy(where, freq.data(), freq.size(), decimation_factor);
}

dft_energy::dft_energy(dft_chunk *E_, dft_chunk *H_, dft_chunk *D_, dft_chunk *B_, const double *freq_, size_t Nfreq,
                       const volume &where_)
    : freq(freq_, freq_ + Nfreq), E(E_), H(H_), D(D_), B(B_), where(where_) {}

// 0.5 sum Re(conj(F1) F2) over the chunk pairs (src/dft.cpp:681-711): the
// real part equals that of F1 conj(F2), the GPU flux reduction
static double *energy_sum(const std::vector<double> &freq, dft_chunk *a, dft_chunk *b) {
  const size_t nf = freq.size();
  double *F = new double[nf];
  for (size_t i = 0; i < nf; i++)
    F[i] = 0;
  std::vector<double> part(nf);
  for (; a && b; a = a->next_in_dft, b = b->next_in_dft) {
    const int ia = a->monitor_id, ib = b->monitor_id;
    chk(mfd_flux(a->fld->d->sim, 1, &ia, &ib, part.data()));
    for (size_t i = 0; i < nf; i++)
      F[i] += 0.5 * part[i];
  }
  return F;
}

double *dft_energy::electric() { return energy_sum(freq, E, D); }
double *dft_energy::magnetic() { return energy_sum(freq, H, B); }

double *dft_energy::total() {
  double *Fe = electric(), *Fm = magnetic();
  for (size_t i = 0; i < freq.size(); i++)
    Fe[i] += Fm[i];
  delete[] Fm;
  return Fe;
}

void dft_energy::scale_dfts(std::complex<double> scale) {
  for (dft_chunk *c : {E, D, H, B})
    if (c) c->scale_dft(scale);
}

/* ------------------------------------------------------------------ LDOS */
// dft_ldos (src/dft_ldos.cpp).  The reference adds E(t) conj(A) over every
// source point to Fdft at each update; here each source's point list gets an
// engine DFT monitor over its bounding box (no weights, the DFT's dt /
// sqrt(2 pi) scale, every step), and ldos() forms sum conj(A) DFT(E) from
// it: the same sum, the E samples at t dt (H at (t - 1/2) dt) with the same
// phases (the t = 0 term of the reference is zero: the fields start at zero).
// Jdft, the DFT of the first source's current, is accumulated on the host at
// each update like the reference's.
dft_ldos::dft_ldos(double freq_min, double freq_max, int Nfreq)
    : freq(linspace(freq_min, freq_max, Nfreq)), Jdft(freq.size(), 0.0) {}
dft_ldos::dft_ldos(const std::vector<double> &freq_) : freq(freq_), Jdft(freq.size(), 0.0) {}
dft_ldos::dft_ldos(const double *freq_, size_t Nfreq) : freq(freq_, freq_ + Nfreq), Jdft(Nfreq, 0.0) {}

void dft_ldos::attach(fields &f) {
  fld = &f;
  ensure_engine(f);
  fields::impl &I = *f.d;
  Dense dn(f.gv);
  Jsum = 0.0;
  for (const PendingSource &ps : I.pending) {
    if (ps.idx.empty()) continue;
    const int t = ps.c / 3, d = ps.c % 3;
    // (sources on D or B components are refused when they are added)
    if (t != MFD_E && t != MFD_H) continue;
    // the field the reference reads for this source: E (or H) along its direction
    const int mc = 3 * t + d;
    int lo[3] = {1 << 30, 1 << 30, 1 << 30}, hi[3] = {-1, -1, -1};
    for (int64_t di : ps.idx) {
      int k[3];
      dn.coords(di, k);
      for (int q = 0; q < 3; q++) {
        lo[q] = std::min(lo[q], k[q]);
        hi[q] = std::max(hi[q], k[q]);
      }
    }
    std::vector<double> ones[3];
    const double *wp[3] = {nullptr, nullptr, nullptr};
    for (int q = 0; q < 3; q++) {
      ones[q].assign(hi[q] - lo[q] + 1, 1.0);
      wp[q] = ones[q].data();
    }
    Mon m;
    chk(mfd_add_dft(I.sim, mc, lo, hi, wp, 1.0, 0, f.dt / std::sqrt(2.0 * pi), 0.0, 0, freq.size(), freq.data(), 1,
                    &m.id));
    for (size_t j = 0; j < ps.idx.size(); j++) {
      int k[3];
      dn.coords(ps.idx[j], k);
      m.at.push_back(((size_t)(k[0] - lo[0]) * (hi[1] - lo[1] + 1) + (k[1] - lo[1])) * (hi[2] - lo[2] + 1) +
                     (k[2] - lo[2]));
      m.amp.push_back(ps.amp[j]);
      Jsum += std::abs(ps.amp[j]);
    }
    mons.push_back(std::move(m));
  }
  // correct for dV factors (src/dft_ldos.cpp:165-166)
  double vol = 1.0;
  LOOP_OVER_DIRECTIONS(f.gv.dim, q) vol *= f.gv.inva;
  Jsum *= std::sqrt(vol);
}

void dft_ldos::check_every_step() const {
  if (skipped)
    meep::abort("dft_ldos::update must run on every step: the engine's DFT of the fields samples every step");
}

void dft_ldos::update(fields &f) {
  if (!fld) attach(f);
  if (fld != &f) meep::abort("dft_ldos updated with another fields object");
  if (last_t >= 0 && f.t > last_t + 1) skipped = true;
  last_t = f.t;
  // the first source's current as the last step left it: its value at the
  // current time (none before the first step)
  if (f.t == 0 || f.d->srcs.empty()) return;
  double cur[2];
  chk(mfd_src_current(f.d->sim, 0, f.time(), cur));
  const std::complex<double> J = f.d->real_fields ? std::complex<double>(cur[0], 0.0) : std::complex<double>(cur[0], cur[1]);
  const double scale = f.dt / std::sqrt(2 * pi);
  for (size_t i = 0; i < freq.size(); ++i) {
    const std::complex<double> Ephase = std::polar(1.0, 2 * pi * freq[i] * f.time()) * scale;
    Jdft[i] += Ephase * J;
  }
}

std::complex<double> *dft_ldos::F() const {
  check_every_step();
  const size_t nf = freq.size();
  std::complex<double> *out = new std::complex<double>[nf];
  for (size_t i = 0; i < nf; i++)
    out[i] = 0.0;
  for (const Mon &m : mons) {
    size_t np = 0, n2 = 0;
    chk(mfd_get_dft(fld->d->sim, m.id, nullptr, &np, &n2));
    std::vector<double> buf(2 * np * nf);
    chk(mfd_get_dft(fld->d->sim, m.id, buf.data(), &np, &n2));
    for (size_t j = 0; j < m.at.size(); j++)
      for (size_t i = 0; i < nf; i++)
        out[i] += std::complex<double>(buf[2 * (m.at[j] * nf + i)], buf[2 * (m.at[j] * nf + i) + 1]) * conj(m.amp[j]);
  }
  return out;
}

std::complex<double> *dft_ldos::J() const {
  check_every_step();
  std::complex<double> *out = new std::complex<double>[freq.size()];
  for (size_t i = 0; i < freq.size(); i++)
    out[i] = Jdft[i];
  return out;
}

// dft_ldos::ldos (src/dft_ldos.cpp:63-86)
double *dft_ldos::ldos() {
  check_every_step();
  saved_overall_scale = 4.0 / pi * -0.5 / (Jsum * Jsum);
  std::complex<double> *Fd = F();
  double *out = new double[freq.size()];
  for (size_t i = 0; i < freq.size(); ++i)
    out[i] = saved_overall_scale * real(Fd[i] * conj(Jdft[i])) /
             (real(Jdft[i]) * real(Jdft[i]) + imag(Jdft[i]) * imag(Jdft[i]));
  delete[] Fd;
  return out;
}

} // namespace meep
