/* meep.hpp -- drop-in C++ API of the GB300 stepping engine.
 *
 * Mirrors the part of the reference's C++ API (src/meep.hpp, src/meep/vec.hpp)
 * that drives the time-stepping path: grid_volume / vec / ivec / volume,
 * material_function, structure (with pml() boundaries, conductivity and
 * Lorentzian/Drude susceptibilities), fields (sources, step(), DFT flux and DFT
 * fields monitors, get_field).  A program written against the reference for
 * this path compiles against this header unchanged, with one extra call when it
 * reads raw DFT chunk arrays: meep::sync_dfts(fields&) copies the device sums
 * into the dft_chunk host buffers.
 *
 * Every field update runs on the GPU through the C ABI in mfd.h.  Names,
 * argument order and meaning follow the reference; errors throw
 * std::runtime_error("meep: ..."), as meep::abort does (src/mympi.cpp:238-254).
 *
 * Precision: realnum is double unless MEEP_SINGLE is defined non-zero, exactly as
 * in the reference (src/meep.hpp:42-46); it selects the engine precision.
 */
#ifndef MEEP_GB300_MEEP_HPP
#define MEEP_GB300_MEEP_HPP

#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#define MEEP_GB300 1

#ifndef MEEP_SINGLE
#define MEEP_SINGLE 0
#endif

struct mfd_sim;

namespace meep {

#if MEEP_SINGLE
typedef float realnum;
#else
typedef double realnum;
#endif

extern int verbosity;
const double pi = 3.141592653589793238462643383276;
const double infinity = HUGE_VAL;
const double nan = NAN;
constexpr int NUM_FIELD_COMPONENTS = 20;

enum component {
  Ex = 0, Ey, Er, Ep, Ez, Hx, Hy, Hr, Hp, Hz, Dx, Dy, Dr, Dp, Dz, Bx, By, Br, Bp, Bz,
  Dielectric, Permeability, NO_COMPONENT
};
const component Centered = Dielectric;
enum derived_component { Sx = 100, Sy, Sr, Sp, Sz, EnergyDensity, D_EnergyDensity, H_EnergyDensity };
enum ndim { D1 = 0, D2, D3, Dcyl };
enum field_type { E_stuff = 0, H_stuff = 1, D_stuff = 2, B_stuff = 3, PE_stuff = 4, PH_stuff = 5,
                  WE_stuff = 6, WH_stuff = 7 };
enum boundary_side { High = 0, Low };
enum direction { X = 0, Y, Z, R, P, NO_DIRECTION };

[[noreturn]] void abort(const char *fmt, ...);
void master_printf(const char *fmt, ...);

inline bool is_electric(component c) { return c < Hx; }
inline bool is_magnetic(component c) { return c >= Hx && c < Dx; }
inline bool is_D(component c) { return c >= Dx && c < Bx; }
inline bool is_B(component c) { return c >= Bx && c < Dielectric; }
inline bool is_E_or_D(component c) { return is_electric(c) || is_D(c); }
inline bool is_H_or_B(component c) { return is_magnetic(c) || is_B(c); }
inline field_type type(component c) {
  if (is_electric(c)) return E_stuff;
  if (is_magnetic(c)) return H_stuff;
  if (is_D(c)) return D_stuff;
  if (is_B(c)) return B_stuff;
  meep::abort("invalid field type");
}
inline direction component_direction(component c) {
  if (c >= Dielectric) return NO_DIRECTION;
  return direction((c % 5) < 2 ? (c % 5) : ((c % 5) == 4 ? Z : ((c % 5) == 2 ? R : P)));
}
inline direction component_direction(derived_component c) {
  switch (c) {
    case Sx: return X;
    case Sy: return Y;
    case Sz: return Z;
    case Sr: return R;
    case Sp: return P;
    default: return NO_DIRECTION;
  }
}
inline component direction_component(component c, direction d) {
  int start = is_electric(c) ? Ex : is_magnetic(c) ? Hx : is_D(c) ? Dx : Bx;
  int off = d == X ? 0 : d == Y ? 1 : d == R ? 2 : d == P ? 3 : 4;
  return component(start + off);
}
inline derived_component direction_component(derived_component c, direction d) {
  (void)c;
  return derived_component(d == X ? Sx : d == Y ? Sy : d == Z ? Sz : d == R ? Sr : Sp);
}
const char *component_name(component c);

inline direction start_at_direction(ndim dim) { return dim == D1 ? Z : (dim == Dcyl ? R : X); }
inline direction stop_at_direction(ndim dim) { return dim == D1 ? R : (dim == D2 ? Z : R); }
#define LOOP_OVER_DIRECTIONS(dim, d)                                                               \
  for (meep::direction d = meep::start_at_direction(dim),                                          \
                       loop_stop_directi = meep::stop_at_direction(dim);                           \
       d < loop_stop_directi; d = (meep::direction)(d + 1))

/* ------------------------------------------------------------- vectors */
class vec {
public:
  ndim dim;
  double t[5];
  vec() : dim(D3) { t[0] = t[1] = t[2] = t[3] = t[4] = 0; }
  explicit vec(ndim di) : dim(di) { t[0] = t[1] = t[2] = t[3] = t[4] = 0; }
  vec(ndim di, double val) : dim(di) { t[0] = t[1] = t[2] = t[3] = t[4] = val; }
  explicit vec(double zz) : dim(D1) {
    t[0] = t[1] = t[2] = t[3] = t[4] = 0;
    t[Z] = zz;
  }
  vec(double xx, double yy) : dim(D2) {
    t[0] = t[1] = t[2] = t[3] = t[4] = 0;
    t[X] = xx;
    t[Y] = yy;
  }
  vec(double xx, double yy, double zz) : dim(D3) {
    t[0] = t[1] = t[2] = t[3] = t[4] = 0;
    t[X] = xx;
    t[Y] = yy;
    t[Z] = zz;
  }
  double x() const { return t[X]; }
  double y() const { return t[Y]; }
  double z() const { return t[Z]; }
  double r() const { return t[R]; }
  double in_direction(direction d) const { return t[d]; }
  void set_direction(direction d, double val) { t[d] = val; }
  vec operator+(const vec &a) const {
    vec r(dim);
    LOOP_OVER_DIRECTIONS(dim, d) r.t[d] = t[d] + a.t[d];
    return r;
  }
  vec operator-(const vec &a) const {
    vec r(dim);
    LOOP_OVER_DIRECTIONS(dim, d) r.t[d] = t[d] - a.t[d];
    return r;
  }
  vec operator-() const {
    vec r(dim);
    LOOP_OVER_DIRECTIONS(dim, d) r.t[d] = -t[d];
    return r;
  }
  vec operator*(double s) const {
    vec r(dim);
    LOOP_OVER_DIRECTIONS(dim, d) r.t[d] = t[d] * s;
    return r;
  }
  vec &operator+=(const vec &a) {
    LOOP_OVER_DIRECTIONS(dim, d) t[d] += a.t[d];
    return *this;
  }
  vec &operator-=(const vec &a) {
    LOOP_OVER_DIRECTIONS(dim, d) t[d] -= a.t[d];
    return *this;
  }
  // multiplies by 1 / s, as the reference's vec does
  vec operator/(double s) const {
    vec r(dim);
    LOOP_OVER_DIRECTIONS(dim, d) r.t[d] = t[d] * (1.0 / s);
    return r;
  }
  // dot product
  double operator&(const vec &a) const {
    double out = 0.0;
    LOOP_OVER_DIRECTIONS(dim, d) out += t[d] * a.t[d];
    return out;
  }
};
inline vec zero_vec(ndim di) { return vec(di, 0.0); }
inline double abs(const vec &v) { return std::sqrt(v & v); }

class ivec {
public:
  ndim dim;
  int t[5];
  ivec() : dim(D3) { t[0] = t[1] = t[2] = t[3] = t[4] = 0; }
  explicit ivec(ndim di) : dim(di) { t[0] = t[1] = t[2] = t[3] = t[4] = 0; }
  ivec(ndim di, int val) : dim(di) { t[0] = t[1] = t[2] = t[3] = t[4] = val; }
  explicit ivec(int zz) : dim(D1) {
    t[0] = t[1] = t[2] = t[3] = t[4] = 0;
    t[Z] = zz;
  }
  ivec(int xx, int yy) : dim(D2) {
    t[0] = t[1] = t[2] = t[3] = t[4] = 0;
    t[X] = xx;
    t[Y] = yy;
  }
  ivec(int xx, int yy, int zz) : dim(D3) {
    t[0] = t[1] = t[2] = t[3] = t[4] = 0;
    t[X] = xx;
    t[Y] = yy;
    t[Z] = zz;
  }
  int x() const { return t[X]; }
  int y() const { return t[Y]; }
  int z() const { return t[Z]; }
  int in_direction(direction d) const { return t[d]; }
  void set_direction(direction d, int val) { t[d] = val; }
  ivec operator+(const ivec &a) const {
    ivec r(dim);
    LOOP_OVER_DIRECTIONS(dim, d) r.t[d] = t[d] + a.t[d];
    return r;
  }
  ivec operator-(const ivec &a) const {
    ivec r(dim);
    LOOP_OVER_DIRECTIONS(dim, d) r.t[d] = t[d] - a.t[d];
    return r;
  }
  ivec operator*(int s) const {
    ivec r(dim);
    LOOP_OVER_DIRECTIONS(dim, d) r.t[d] = t[d] * s;
    return r;
  }
  vec operator*(double s) const {
    vec r(dim);
    LOOP_OVER_DIRECTIONS(dim, d) r.t[d] = t[d] * s;
    return r;
  }
  ivec &operator+=(const ivec &a) {
    LOOP_OVER_DIRECTIONS(dim, d) t[d] += a.t[d];
    return *this;
  }
  bool operator==(const ivec &a) const {
    LOOP_OVER_DIRECTIONS(dim, d) if (t[d] != a.t[d]) return false;
    return true;
  }
  bool operator!=(const ivec &a) const { return !(*this == a); }
  bool operator<=(const ivec &a) const {
    LOOP_OVER_DIRECTIONS(dim, d) if (t[d] > a.t[d]) return false;
    return true;
  }
};
inline ivec zero_ivec(ndim di) { return ivec(di, 0); }
inline ivec one_ivec(ndim di) {
  ivec r(di, 0);
  LOOP_OVER_DIRECTIONS(di, d) r.t[d] = 1;
  return r;
}
inline ivec max(const ivec &a, const ivec &b) {
  ivec r(a.dim);
  LOOP_OVER_DIRECTIONS(a.dim, d) r.t[d] = a.t[d] > b.t[d] ? a.t[d] : b.t[d];
  return r;
}
inline ivec min(const ivec &a, const ivec &b) {
  ivec r(a.dim);
  LOOP_OVER_DIRECTIONS(a.dim, d) r.t[d] = a.t[d] < b.t[d] ? a.t[d] : b.t[d];
  return r;
}

class volume {
public:
  ndim dim;
  vec min_corner, max_corner;
  explicit volume(ndim di) : dim(di), min_corner(di), max_corner(di) {}
  volume(const vec &vec1, const vec &vec2);
  explicit volume(const vec &pt) : volume(pt, pt) {}
  vec get_min_corner() const { return min_corner; }
  vec get_max_corner() const { return max_corner; }
  double in_direction_min(direction d) const { return min_corner.in_direction(d); }
  double in_direction_max(direction d) const { return max_corner.in_direction(d); }
  double in_direction(direction d) const { return max_corner.in_direction(d) - min_corner.in_direction(d); }
  void set_direction_min(direction d, double v) { min_corner.set_direction(d, v); }
  void set_direction_max(direction d, double v) { max_corner.set_direction(d, v); }
  vec center() const { return (min_corner + max_corner) * 0.5; }
  volume operator+(const vec &a) const { return volume(min_corner + a, max_corner + a); }
  // smallest volume containing both
  volume operator|(const volume &a) const;
};

class grid_volume {
public:
  ndim dim;
  double a, inva;
  grid_volume() : dim(D3), a(1), inva(1), io(D3), origin(D3) { num[0] = num[1] = num[2] = 0; }
  grid_volume(ndim td, double ta, int na, int nb, int nc);
  int nx() const { return num[0]; }
  int ny() const { return num[1]; }
  int nz() const { return num[2]; }
  int num_direction(direction d) const { return d == X ? num[0] : d == Y ? num[1] : d == Z ? num[2] : 0; }
  ivec little_corner() const { return io; }
  ivec big_corner() const;
  ivec iyee_shift(component c) const;
  vec yee_shift(component c) const { return operator[](iyee_shift(c)); }
  vec operator[](const ivec &p) const { return p * (0.5 * inva); }
  vec center() const { return operator[](icenter()); }
  ivec icenter() const;
  void center_origin() {
    ivec s = icenter();
    set_origin(io - s);
  }
  void set_origin(const ivec &o);
  void shift_origin(const ivec &s) { set_origin(io + s); }
  ivec little_owned_corner(component c) const { return little_corner() + one_ivec(dim) * 2 - iyee_shift(c); }
  ivec big_owned_corner(component c) const { return big_corner() - iyee_shift(c); }
  bool owns(const ivec &p) const;
  bool has_field(component c) const {
    if (dim == D1) return c == Ex || c == Hy || c == Dx || c == By;
    return c < Dielectric && component_direction(c) < R;
  }
  volume surroundings() const { return volume(operator[](little_corner()), operator[](big_corner())); }
  double boundary_location(boundary_side b, direction d) const;
  size_t ntot() const;

private:
  int num[3];
  ivec io;
  vec origin;
};
grid_volume volone(double zsize, double a);
grid_volume vol1d(double zsize, double a);
grid_volume voltwo(double xsize, double ysize, double a);
grid_volume vol2d(double xsize, double ysize, double a);
grid_volume vol3d(double xsize, double ysize, double zsize, double a);

class symmetry {
public:
  symmetry() {}
};
symmetry identity();

/* ---------------------------------------------------------- boundaries */
class boundary_region {
public:
  enum boundary_region_kind { NOTHING_SPECIAL, PML };
  struct part {
    boundary_region_kind kind;
    double thickness, Rasymptotic, mean_stretch;
    direction d;
    boundary_side side;
  };
  std::vector<part> parts;
  boundary_region() {}
  boundary_region(boundary_region_kind kind, double thickness, double Rasymptotic,
                  double mean_stretch, direction d, boundary_side side) {
    parts.push_back({kind, thickness, Rasymptotic, mean_stretch, d, side});
  }
  boundary_region operator+(const boundary_region &r0) const {
    boundary_region r = *this;
    r.parts.insert(r.parts.end(), r0.parts.begin(), r0.parts.end());
    return r;
  }
};
boundary_region pml(double thickness, direction d, boundary_side side, double Rasymptotic = 1e-15,
                    double mean_stretch = 1.0);
boundary_region pml(double thickness, direction d, double Rasymptotic = 1e-15,
                    double mean_stretch = 1.0);
boundary_region pml(double thickness, double Rasymptotic = 1e-15, double mean_stretch = 1.0);

/* ----------------------------------------------------------- materials */
#define DEFAULT_SUBPIXEL_TOL 1e-4
#define DEFAULT_SUBPIXEL_MAXEVAL 100000

class material_function {
public:
  material_function() {}
  virtual ~material_function() {}
  virtual void set_volume(const volume &v) { (void)v; }
  virtual void unset_volume(void) {}
  virtual double chi1p1(field_type ft, const vec &r) {
    (void)ft;
    (void)r;
    return 1.0;
  }
  virtual double eps(const vec &r) { return chi1p1(E_stuff, r); }
  virtual bool has_mu() { return false; }
  virtual double mu(const vec &r) { return chi1p1(H_stuff, r); }
  virtual bool has_conductivity(component c) {
    (void)c;
    return false;
  }
  virtual double conductivity(component c, const vec &r) {
    (void)c;
    (void)r;
    return 0.0;
  }
  // Gradient of chi1p1 over the pixel v by a sphere quadrature, zero where
  // the material is uniform (src/anisotropic_averaging.cpp:60-85).
  vec normal_vector(field_type ft, const volume &v);
  // Effective inverse-permittivity row of the pixel v: 1/chi1p1 at its centre
  // when maxeval == 0 or the material is uniform there, else the averaged
  // tensor row (src/anisotropic_averaging.cpp:87-208).
  virtual void eff_chi1inv_row(component c, double chi1inv_row[3], const volume &v,
                               double tol = DEFAULT_SUBPIXEL_TOL,
                               int maxeval = DEFAULT_SUBPIXEL_MAXEVAL);
  virtual bool is_thread_safe() const { return false; }
  // Extension of this engine, not in the reference: the rows of n pixels at
  // once (lo, hi: n x 3 pixel corners in x, y, z order; rows: n x 3).  A
  // material that evaluates them in bulk (on the GPU) returns true; the
  // default returns false and the structure calls eff_chi1inv_row per pixel.
  virtual bool eff_chi1inv_rows(component c, size_t n, const double *lo, const double *hi, double tol,
                                int maxeval, double *rows) {
    (void)c, (void)n, (void)lo, (void)hi, (void)tol, (void)maxeval, (void)rows;
    return false;
  }
  virtual void sigma_row(component c, double sigrow[3], const vec &r) {
    (void)c;
    (void)r;
    sigrow[0] = sigrow[1] = sigrow[2] = 0.0;
  }
  virtual bool has_chi3(component c) {
    (void)c;
    return false;
  }
  virtual bool has_chi2(component c) {
    (void)c;
    return false;
  }
};

class simple_material_function : public material_function {
  double (*f)(const vec &);

public:
  explicit simple_material_function(double (*func)(const vec &)) : f(func) {}
  double chi1p1(field_type ft, const vec &r) override {
    (void)ft;
    return f(r);
  }
  double eps(const vec &r) override { return f(r); }
  double mu(const vec &r) override { return f(r); }
  double conductivity(component c, const vec &r) override {
    (void)c;
    return f(r);
  }
  void sigma_row(component c, double sigrow[3], const vec &r) override {
    sigrow[0] = sigrow[1] = sigrow[2] = 0.0;
    sigrow[component_direction(c) % 3] = f(r);
  }
};

class susceptibility {
public:
  virtual ~susceptibility() {}
  virtual susceptibility *clone() const = 0;
};

class lorentzian_susceptibility : public susceptibility {
public:
  double omega_0, gamma;
  bool no_omega_0_denominator;
  lorentzian_susceptibility(double omega_0, double gamma, bool no_omega_0_denominator = false)
      : omega_0(omega_0), gamma(gamma), no_omega_0_denominator(no_omega_0_denominator) {}
  susceptibility *clone() const override { return new lorentzian_susceptibility(*this); }
};

class drude_susceptibility : public lorentzian_susceptibility {
public:
  drude_susceptibility(double omega_0, double gamma) : lorentzian_susceptibility(omega_0, gamma, true) {}
};

class fields;

class structure {
public:
  grid_volume gv, user_volume;
  double a, Courant, dt;
  boundary_region br;

  structure(const grid_volume &gv, material_function &eps,
            const boundary_region &br = boundary_region(), const symmetry &s = meep::identity(),
            int num_chunks = 0, double Courant = 0.5, bool use_anisotropic_averaging = false,
            double tol = DEFAULT_SUBPIXEL_TOL, int maxeval = DEFAULT_SUBPIXEL_MAXEVAL);
  structure(const grid_volume &gv, double eps(const vec &),
            const boundary_region &br = boundary_region(), const symmetry &s = meep::identity(),
            int num_chunks = 0, double Courant = 0.5, bool use_anisotropic_averaging = false,
            double tol = DEFAULT_SUBPIXEL_TOL, int maxeval = DEFAULT_SUBPIXEL_MAXEVAL);
  ~structure();

  void set_materials(material_function &mat, bool use_anisotropic_averaging = true,
                     double tol = DEFAULT_SUBPIXEL_TOL, int maxeval = DEFAULT_SUBPIXEL_MAXEVAL);
  void set_epsilon(material_function &eps, bool use_anisotropic_averaging = true,
                   double tol = DEFAULT_SUBPIXEL_TOL, int maxeval = DEFAULT_SUBPIXEL_MAXEVAL);
  void set_epsilon(double eps(const vec &), bool use_anisotropic_averaging = true,
                   double tol = DEFAULT_SUBPIXEL_TOL, int maxeval = DEFAULT_SUBPIXEL_MAXEVAL);
  // inverse-permittivity tensor entry (c, d) at a grid point owned by the
  // cell (frequency 0 only); 0 elsewhere (src/monitor.cpp:196-212)
  std::complex<double> get_chi1inv(component c, direction d, const ivec &origloc, double frequency = 0,
                                   bool parallel = true) const;
  std::complex<double> get_inveps(component c, direction d, const ivec &origloc, double frequency = 0) const {
    return get_chi1inv(c, d, origloc, frequency);
  }
  void set_conductivity(component c, material_function &conductivity);
  void set_conductivity(component c, double Cfunc(const vec &));
  void add_susceptibility(material_function &sigma, field_type ft, const susceptibility &sus);
  void add_susceptibility(double sigma(const vec &), field_type ft, const susceptibility &sus);
  // Extension (the reference reaches material grids through its libctl
  // geometry, src/meepgeom.cpp:489-581): a material grid over the axis-
  // aligned block (center, size), weights u (n[0] x n[1] x n[2], row-major),
  // projection (beta, eta), eps = eps1 + p (eps2 - eps1) per direction.  The
  // engine evaluates it on the device over the E components' diagonal
  // chi1inv when the fields are created, after the other materials.
  void add_material_grid(const double center[3], const double size[3], const int n[3], const double *weights,
                         double beta, double eta, const double eps1[3], const double eps2[3]);

  // host copies handed to the engine when fields are created
  struct impl;
  std::unique_ptr<impl> d;
};

/* ------------------------------------------------------------- sources */
class src_time {
public:
  bool is_integrated;
  src_time() : is_integrated(true) {}
  virtual ~src_time() {}
  virtual src_time *clone() const = 0;
  virtual int kind() const = 0;
  virtual std::complex<double> frequency() const = 0;
  virtual double get_fwidth() const = 0;
  virtual double last_time() const { return 0.0; }
  // parameters forwarded to the engine (see mfd_add_*_src)
  double p[6] = {0, 0, 0, 0, 0, 0};
};

class gaussian_src_time : public src_time {
public:
  gaussian_src_time(double f, double fwidth, double s = 5.0);
  gaussian_src_time(double f, double w, double start_time, double end_time);
  src_time *clone() const override { return new gaussian_src_time(*this); }
  int kind() const override { return 0; }
  std::complex<double> frequency() const override { return freq; }
  double get_fwidth() const override { return fwidth; }
  double last_time() const override { return float(peak_time + cutoff); }
  double freq, fwidth, width, peak_time, cutoff;
  bool explicit_window;
};

class continuous_src_time : public src_time {
public:
  continuous_src_time(std::complex<double> f, double w = 0.0, double st = 0.0,
                      double et = infinity, double s = 3.0);
  src_time *clone() const override { return new continuous_src_time(*this); }
  int kind() const override { return 1; }
  std::complex<double> frequency() const override { return freq; }
  double get_fwidth() const override { return 0.0; }
  double last_time() const override { return end_time; }
  std::complex<double> freq;
  double width, start_time, end_time, slowness;
};

/* ------------------------------------------------------------ monitors */
class fields;

class dft_chunk {
public:
  std::vector<double> omega;
  component c;
  size_t N;
  std::complex<realnum> *dft;
  dft_chunk *next_in_dft;
  ivec is, ie;
  ivec shift; // lattice-image shift of the chunk's points
  int vc;     // equivalent source component (near2far), else c
  int monitor_id;
  fields *fld;
  std::complex<double> extra_weight; // weight of the force sum (dft_force)
  int decimation_factor;             // steps between accumulated samples (src/meep.hpp:1196)
  dft_chunk()
      : c(Ex), N(0), dft(nullptr), next_in_dft(nullptr), vc(Ex), monitor_id(-1), fld(nullptr),
        extra_weight(1.0), decimation_factor(1) {}
  int get_decimation_factor() const { return decimation_factor; }
  ~dft_chunk() { delete[] dft; }
  // multiply the sums of this chunk and the chunks after it (device sums)
  void scale_dft(std::complex<double> scale);
};

class volume_list {
public:
  volume v;
  int c; // component or derived_component
  std::complex<double> weight;
  volume_list *next;
  volume_list(const volume &v, int c, std::complex<double> weight = 1.0, volume_list *next = 0)
      : v(v), c(c), weight(weight), next(next) {}
  ~volume_list() { delete next; }
};

class dft_flux {
public:
  std::vector<double> freq;
  dft_chunk *E, *H;
  component cE, cH;
  fields *f;
  dft_flux() : E(nullptr), H(nullptr), cE(Ex), cH(Hy), f(nullptr) {}
  double *flux();
  void scale_dfts(std::complex<double> scale);
};

// the DFT sums of a chunk list as one array, chunk after chunk (the layout
// of the reference's Python get_dft_data / load_dft_data helpers)
size_t dft_data_size(dft_chunk *chunks);
void get_dft_data(dft_chunk *chunks, std::complex<double> *data, size_t n);
void load_dft_data(dft_chunk *chunks, const std::complex<double> *data, size_t n);

/* Near-to-far transform (src/near2far.cpp): DFT chunks of the tangential
   fields on closed or open surfaces in a homogeneous medium; far fields by
   the 2-D or 3-D Green's function, evaluated on the GPU. */
class dft_near2far {
public:
  dft_near2far(dft_chunk *F, const double *freq, size_t Nfreq, double eps, double mu, const volume &where,
               const direction periodic_d[2], const int periodic_n[2], const double periodic_k[2],
               const double period[2]);
  // (Ex, Ey, Ez, Hx, Hy, Hz) x Nfreq at x, newly allocated
  std::complex<double> *farfield(const vec &x, double greencyl_tol = 1e-3);
  // the same into a caller array of 6 * Nfreq values
  void farfield_lowlevel(std::complex<double> *EH, const vec &x, double greencyl_tol = 1e-3);
  // 6 x 2 x N x Nfreq fields on a grid over `where` at `resolution`
  double *get_farfields_array(const volume &where, int &rank, size_t *dims, size_t &N, double resolution,
                              double greencyl_tol = 1e-3);
  // Poynting flux through `where` (normal df) of the far fields
  double *flux(direction df, const volume &where, double resolution);
  void scale_dfts(std::complex<double> scale);
  void remove();
  // the far fields at many points in one engine call (an extension): out
  // has npts * Nfreq * 6 values, point-major like farfield's result
  void farfields_at(const std::vector<vec> &pts, std::complex<double> *out);

  std::vector<double> freq;
  dft_chunk *F;
  double eps, mu;
  volume where;
  direction periodic_d[2];
  int periodic_n[2];
  double periodic_k[2], period[2];
};

// local density of states of the sources (src/dft_ldos.cpp): call
// update(f) before every step and once after the last, as the reference's
// dft_ldos step function does
class dft_ldos {
public:
  dft_ldos(double freq_min, double freq_max, int Nfreq);
  explicit dft_ldos(const std::vector<double> &freq);
  dft_ldos(const double *freq, size_t Nfreq);
  void update(fields &f);
  double *ldos();                   // newly allocated, Nfreq values
  std::complex<double> *F() const; // the DFT of sum E conj(J) (and H)
  std::complex<double> *J() const; // the DFT of the first source's current
  double overall_scale() const { return saved_overall_scale; }
  std::vector<double> freq;

private:
  struct Mon {
    int id;                      // engine DFT monitor over the points' box
    std::vector<size_t> at;      // each point's index in the monitor box
    std::vector<std::complex<double>> amp;
  };
  fields *fld = nullptr;
  std::vector<Mon> mons;
  std::vector<std::complex<double>> Jdft;
  double Jsum = 1.0, saved_overall_scale = 1.0;
  // the engine's monitors sample every step, so update() must run on every
  // step for F and J to hold the same samples (checked in F, J and ldos)
  long long last_t = -1;
  bool skipped = false;
  void attach(fields &f);
  void check_every_step() const;
};

// electric and magnetic energy density spectra in volumes (src/dft.cpp
// dft_energy): created by fields::add_dft_energy
class dft_energy {
public:
  dft_energy(dft_chunk *E, dft_chunk *H, dft_chunk *D, dft_chunk *B, const double *freq, size_t Nfreq,
             const volume &where);
  double *electric(); // newly allocated, Nfreq values
  double *magnetic();
  double *total();
  void scale_dfts(std::complex<double> scale);
  std::vector<double> freq;
  dft_chunk *E, *H, *D, *B;
  volume where;
};

// Maxwell-stress force on surfaces (src/stress.cpp): created by
// fields::add_dft_force
class dft_force {
public:
  dft_force(dft_chunk *offdiag1, dft_chunk *offdiag2, dft_chunk *diag, const double *freq, size_t Nfreq,
            const volume &where);
  double *force(); // newly allocated, Nfreq values
  void scale_dfts(std::complex<double> scale);
  std::vector<double> freq;
  dft_chunk *offdiag1, *offdiag2, *diag;
  volume where;
};

// homogeneous-medium Green's functions (src/near2far.cpp:131-245), on the GPU
void green3d(std::complex<double> *EH, const vec &x, double freq, double eps, double mu, const vec &x0,
             component c0, std::complex<double> f0);
void green2d(std::complex<double> *EH, const vec &x, double freq, double eps, double mu, const vec &x0,
             component c0, std::complex<double> f0);

class dft_fields {
public:
  std::vector<double> freq;
  dft_chunk *chunks;
  volume where;
  dft_fields(dft_chunk *chunks, const std::vector<double> &freq, const volume &where)
      : freq(freq), chunks(chunks), where(where) {}
};

std::vector<double> linspace(double freq_min, double freq_max, size_t Nfreq);

class fields {
public:
  int t;
  double dt, a;
  grid_volume gv, user_volume;
  structure *s;

  explicit fields(structure *s, double m = 0, double beta = 0,
                  bool zero_fields_near_cylorigin = true, int loop_tile_base_db = 0,
                  int loop_tile_base_eh = 0);
  ~fields();

  void use_real_fields();
  void use_bloch(direction d, double k);
  void use_bloch(const vec &k);
  void step();
  double time() const { return t * dt; }
  // latest time any source is still on (src/bands.cpp:35-41)
  double last_source_time() const;
  double round_time() const { return float(t * dt); }
  double last_step_ms() const;
  long long kernel_launches() const;

  void add_point_source(component c, double freq, double width, double peaktime, double cutoff,
                        const vec &p, std::complex<double> amp = 1.0, int is_continuous = 0);
  void add_point_source(component c, const src_time &src, const vec &p,
                        std::complex<double> amp = 1.0);
  void add_volume_source(component c, const src_time &src, const volume &where,
                         std::complex<double> A(const vec &), std::complex<double> amp = 1.0);
  void add_volume_source(component c, const src_time &src, const volume &where,
                         std::complex<double> amp = 1.0);

  dft_flux add_dft_flux(const volume_list *where, const double *freq, size_t Nfreq,
                        bool use_symmetry = true, bool centered_grid = true,
                        int decimation_factor = 0);
  dft_flux add_dft_flux(direction d, const volume &where, double freq_min, double freq_max,
                        int Nfreq, bool use_symmetry = true, bool centered_grid = true,
                        int decimation_factor = 0);
  dft_flux add_dft_flux(direction d, const volume &where, const std::vector<double> &freq,
                        bool use_symmetry = true, bool centered_grid = true,
                        int decimation_factor = 0);
  dft_flux add_dft_flux_plane(const volume &where, double freq_min, double freq_max, int Nfreq);
  dft_fields add_dft_fields(component *components, int num_components, const volume where,
                            const double *freq, size_t Nfreq, bool use_centered_grid = true,
                            int decimation_factor = 0, bool persist = false);
  dft_fields add_dft_fields(component *components, int num_components, const volume where,
                            double freq_min, double freq_max, int Nfreq,
                            bool use_centered_grid = true, int decimation_factor = 0,
                            bool persist = false);

  dft_near2far add_dft_near2far(const volume_list *where, double freq_min, double freq_max, int Nfreq,
                                int decimation_factor = 0, int Nperiods = 1);
  dft_near2far add_dft_near2far(const volume_list *where, const std::vector<double> &freq,
                                int decimation_factor = 0, int Nperiods = 1);
  dft_near2far add_dft_near2far(const volume_list *where, const double *freq, size_t Nfreq,
                                int decimation_factor = 0, int Nperiods = 1);
  dft_energy add_dft_energy(const volume_list *where, double freq_min, double freq_max, int Nfreq,
                            int decimation_factor = 0);
  dft_energy add_dft_energy(const volume_list *where, const std::vector<double> &freq, int decimation_factor = 0);
  dft_energy add_dft_energy(const volume_list *where, const double *freq, size_t Nfreq, int decimation_factor = 0);
  dft_force add_dft_force(const volume_list *where, double freq_min, double freq_max, int Nfreq,
                          int decimation_factor = 0);
  dft_force add_dft_force(const volume_list *where, const std::vector<double> &freq, int decimation_factor = 0);
  dft_force add_dft_force(const volume_list *where, const double *freq, size_t Nfreq, int decimation_factor = 0);
  // trace-averaged permittivity / permeability at loc (src/monitor.cpp:172-194)
  std::complex<double> get_eps(const vec &loc, double frequency = 0) const;
  std::complex<double> get_mu(const vec &loc, double frequency = 0) const;

  std::complex<double> get_field(component c, const vec &loc, bool parallel = true);
  std::complex<double> get_field(component c, const ivec &iloc, bool parallel = true);
  // dense host copy of component c (x slowest), as in mfd_get_field
  std::vector<double> get_field_array(component c);

  // internal
  struct impl;
  std::unique_ptr<impl> d;
  void sync_dfts();
};

// Copy the device DFT sums into the host dft_chunk::dft buffers.
void sync_dfts(fields &f);
// Advance n steps in one batched engine call (same result as n calls of step()).
void step_n(fields &f, int n);

class initialize {
public:
  initialize(int &argc, char **&argv) {
    (void)argc;
    (void)argv;
  }
};

} // namespace meep

#endif
