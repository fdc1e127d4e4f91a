// C interface of the meep:: drop-in for the Python Simulation front end
// (declarations and contract: include/meep_gb300/mgb.h).
//
// Mirrors what the reference's Python layer asks of its C++ core:
//   Simulation._init_structure / _create_grid_volume  python/simulation.py
//     vol1d/vol2d/vol3d + center_origin, boundary_region from PML layers
//   geom_epsilon (libctl geometry as a material_function)  src/meepgeom.cpp
//     material of the last object containing the point, else the default;
//     chi1inv = 1 / epsilon_diag at the pixel centre without averaging;
//     D conductivity; one polarization per distinct susceptibility with the
//     sigma of the material at the point
//   Source.add_source -> fields::add_volume_source   python/source.py
//   Simulation._add_fluxish_stuff -> add_dft_flux(volume_list, ...)
//   Simulation._add_dft_fields -> add_dft_fields(...)
#include <cmath>
#include <complex>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "meep.hpp"
#include "mfd.h"
#include "mgb.h"
#include "geom_eval.hpp"

using namespace meep;

namespace {

thread_local std::string g_err;

struct Geometry {
  int dim = 3;
  std::vector<mgb_object> objs;
  std::vector<mgb_medium> media;
  int def = 0;

  static double coord(const vec &r, int d, int dim) {
    if (dim == 1) return d == 2 ? r.z() : 0.0;
    if (dim == 2) return d == 0 ? r.x() : (d == 1 ? r.y() : 0.0);
    return d == 0 ? r.x() : (d == 1 ? r.y() : r.z());
  }
  bool inside(const mgb_object &o, const vec &r) const {
    const double p[3] = {coord(r, 0, dim), coord(r, 1, dim), coord(r, 2, dim)};
    return mgb_geom::contains(o, p);
  }
  const mgb_medium &at(const vec &r) const {
    for (size_t q = objs.size(); q-- > 0;)
      if (inside(objs[q], r)) return media[objs[q].material];
    return media[def];
  }
};

class GeomMaterial : public material_function {
public:
  const Geometry *g;
  std::vector<mfd_object> dev; // the objects with their scalar permittivity
  explicit GeomMaterial(const Geometry *geo) : g(geo) {
    for (const mgb_object &o : g->objs) {
      mfd_object m{};
      m.kind = o.kind;
      for (int d = 0; d < 3; d++) {
        m.center[d] = o.center[d];
        m.size[d] = o.size[d];
        m.axis[d] = o.axis[d];
      }
      m.radius = o.radius;
      m.height = o.height;
      m.eps = g->media[o.material].eps[0];
      dev.push_back(m);
    }
  }
  bool isotropic() const {
    for (const mgb_medium &m : g->media)
      if (m.eps[1] != m.eps[0] || m.eps[2] != m.eps[0]) return false;
    return true;
  }
  double chi1p1(field_type ft, const vec &r) override { return ft == H_stuff ? 1.0 : g->at(r).eps[0]; }
  // without averaging: 1 / epsilon_diag at the pixel centre; with averaging
  // (isotropic media): the default material_function averaging
  void eff_chi1inv_row(component c, double row[3], const volume &v, double tol, int maxeval) override {
    if (maxeval && type(c) == E_stuff) {
      if (!isotropic()) meep::abort("subpixel averaging of anisotropic media is not supported by the GB300 engine");
      material_function::eff_chi1inv_row(c, row, v, tol, maxeval);
      return;
    }
    row[0] = row[1] = row[2] = 0.0;
    const int d = component_direction(c) % 3;
    if (type(c) == H_stuff) {
      row[d] = 1.0;
      return;
    }
    row[d] = 1.0 / g->at(v.center()).eps[d];
  }
  // averaged rows of many pixels at once on the GPU (mfd_subpixel_rows)
  bool eff_chi1inv_rows(component c, size_t n, const double *lo, const double *hi, double tol, int maxeval,
                        double *rows) override {
    if (!maxeval || type(c) != E_stuff) return false;
    if (!isotropic()) meep::abort("subpixel averaging of anisotropic media is not supported by the GB300 engine");
    if (mfd_subpixel_rows(g->dim, component_direction(c) % 3, (int64_t)n, lo, hi, tol, maxeval, (int)dev.size(),
                          dev.data(), g->media[g->def].eps[0], rows) != 0)
      throw std::runtime_error(mfd_last_error());
    return true;
  }
  bool is_thread_safe() const override { return true; }
  bool has_conductivity(component c) override {
    if (!is_D(c)) return false;
    const int d = component_direction(c) % 3;
    for (const mgb_medium &m : g->media)
      if (m.d_cond[d] != 0.0) return true;
    return false;
  }
  double conductivity(component c, const vec &r) override { return g->at(r).d_cond[component_direction(c) % 3]; }
};

// sigma of susceptibility q: the material's sigma_diag where it has q
class SusSigma : public material_function {
public:
  const Geometry *g;
  int q;
  SusSigma(const Geometry *geo, int idx) : g(geo), q(idx) {}
  bool is_thread_safe() const override { return true; }
  void sigma_row(component c, double row[3], const vec &r) override {
    row[0] = row[1] = row[2] = 0.0;
    const mgb_medium &m = g->at(r);
    const int d = component_direction(c) % 3;
    for (int k = 0; k < m.nsus && k < MGB_MAX_SUS; k++)
      if (m.sus[k] == q) row[d] = m.sigma[k][d];
  }
};

vec mkvec(int dim, const double p[3]) {
  if (dim == 1) return vec(p[2]);
  if (dim == 2) return vec(p[0], p[1]);
  return vec(p[0], p[1], p[2]);
}

volume mkvol(int dim, const double c[3], const double s[3]) {
  double lo[3], hi[3];
  for (int d = 0; d < 3; d++) {
    lo[d] = c[d] - 0.5 * s[d];
    hi[d] = c[d] + 0.5 * s[d];
  }
  return volume(mkvec(dim, lo), mkvec(dim, hi));
}

int fail(const std::exception &e) {
  g_err = e.what();
  if (g_err.rfind("meep:", 0) != 0) g_err = "meep: " + g_err;
  return -1;
}

} // namespace

struct mgb_sim {
  int dim = 3;
  Geometry geo;
  std::unique_ptr<GeomMaterial> mat;
  std::vector<std::unique_ptr<SusSigma>> sigmas;
  grid_volume gv;
  std::unique_ptr<structure> s;
  std::unique_ptr<fields> f;
  std::vector<std::unique_ptr<src_time>> srcs;
  std::vector<dft_flux> fluxes;
  std::vector<dft_fields> dfts;
  std::vector<dft_near2far> n2fs;
  std::vector<dft_force> forces;
  std::vector<dft_energy> energies;
  std::vector<std::unique_ptr<dft_ldos>> ldoses;
};

// rows of (center[3], size[3], direction or -1, weight) as a volume_list;
// regions are prepended, as the Python layer builds its volume_list
static std::unique_ptr<volume_list> region_list(mgb_sim *s, int nreg, const double *regions) {
  std::unique_ptr<volume_list> head;
  for (int q = 0; q < nreg; q++) {
    const double *r = regions + 8 * q;
    volume v = mkvol(s->dim, r, r + 3);
    int d = (int)r[6];
    if (d < 0) {
      // fields::normal_direction: the one present direction of zero extent
      int nzero = 0;
      for (int dd = 0; dd < 3; dd++) {
        if ((s->dim == 1 && dd != 2) || (s->dim == 2 && dd == 2)) continue;
        if (r[3 + dd] == 0.0) {
          d = dd;
          nzero++;
        }
      }
      if (nzero != 1) throw std::runtime_error("meep: flux region needs a normal direction");
    }
    head.reset(new volume_list(v, (int)direction_component(Sx, (direction)d), r[7], head.release()));
  }
  return head;
}

extern "C" {

const char *mgb_last_error(void) { return g_err.c_str(); }

int mgb_create(int dim, const double cell[3], double resolution, double courant, int npml, const double *pmlspec,
               int nmed, const mgb_medium *media, int default_medium, int nobj, const mgb_object *objects,
               int nsus, const mgb_susceptibility *sus, int eps_averaging, double subpixel_tol,
               int subpixel_maxeval, mgb_sim **out) {
  try {
    if (!out || !cell || (nmed > 0 && !media)) throw std::runtime_error("null argument");
    if (dim < 1 || dim > 3) throw std::runtime_error("dimensions must be 1, 2 or 3");
    if (nmed < 1 || default_medium < 0 || default_medium >= nmed) throw std::runtime_error("bad medium table");
    std::unique_ptr<mgb_sim> S(new mgb_sim);
    S->dim = dim;
    S->geo.dim = dim;
    S->geo.media.assign(media, media + nmed);
    S->geo.objs.assign(objects, objects + nobj);
    S->geo.def = default_medium;
    for (const mgb_object &o : S->geo.objs)
      if (o.material < 0 || o.material >= nmed) throw std::runtime_error("object material out of range");
    if (dim == 1) S->gv = vol1d(cell[2], resolution);
    else if (dim == 2) S->gv = vol2d(cell[0], cell[1], resolution);
    else S->gv = vol3d(cell[0], cell[1], cell[2], resolution);
    S->gv.center_origin();
    boundary_region br;
    for (int q = 0; q < npml; q++) {
      const double *r = pmlspec + 5 * q;
      const int d = (int)r[1], side = (int)r[2];
      for (int dd = 0; dd < 3; dd++) {
        if (d >= 0 && dd != d) continue;
        if (dim == 1 && dd != 2) continue;
        if (dim == 2 && dd == 2) continue;
        if (side < 0) br = br + pml(r[0], (direction)dd, r[3], r[4]);
        else br = br + pml(r[0], (direction)dd, (boundary_side)side, r[3], r[4]);
      }
    }
    S->mat.reset(new GeomMaterial(&S->geo));
    S->s.reset(new structure(S->gv, *S->mat, br, identity(), 0, courant, eps_averaging != 0, subpixel_tol,
                             subpixel_maxeval));
    for (int q = 0; q < nsus; q++) {
      S->sigmas.emplace_back(new SusSigma(&S->geo, q));
      // Drude: the Lorentzian without the omega_0^2 term (src/meepgeom.cpp)
      S->s->add_susceptibility(*S->sigmas.back(), E_stuff,
                               lorentzian_susceptibility(sus[q].frequency, sus[q].gamma, sus[q].drude != 0));
    }
    S->f.reset(new fields(S->s.get()));
    *out = S.release();
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

void mgb_destroy(mgb_sim *s) { delete s; }

int mgb_add_source(mgb_sim *s, int component_, int kind, const double *p, int is_integrated,
                   const double center[3], const double size[3], double amp_re, double amp_im) {
  try {
    if (!s || !p || !center || !size) throw std::runtime_error("null argument");
    std::unique_ptr<src_time> st;
    if (kind == 0) st.reset(new gaussian_src_time(p[0], p[1], p[2], p[3]));
    else if (kind == 1) st.reset(new continuous_src_time(p[0], p[1], p[2], p[3], p[4]));
    else throw std::runtime_error("unknown source time kind");
    st->is_integrated = is_integrated != 0;
    s->f->add_volume_source((component)component_, *st, mkvol(s->dim, center, size),
                            std::complex<double>(amp_re, amp_im));
    s->srcs.push_back(std::move(st));
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

double mgb_last_source_time(const mgb_sim *s) { return s ? s->f->last_source_time() : 0.0; }

int mgb_add_flux(mgb_sim *s, int nreg, const double *regions, int nfreq, const double *freqs, int decimation,
                 int *handle) {
  try {
    if (!s || !regions || !freqs || !handle || nreg < 1) throw std::runtime_error("null argument");
    std::unique_ptr<volume_list> head = region_list(s, nreg, regions);
    s->fluxes.push_back(s->f->add_dft_flux(head.get(), freqs, (size_t)nfreq, true, true, decimation));
    *handle = (int)s->fluxes.size() - 1;
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_flux(mgb_sim *s, int handle, double *out) {
  try {
    if (!s || !out || handle < 0 || handle >= (int)s->fluxes.size()) throw std::runtime_error("bad flux handle");
    double *F = s->fluxes[handle].flux();
    for (size_t i = 0; i < s->fluxes[handle].freq.size(); i++)
      out[i] = F[i];
    delete[] F;
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

// the chunk lists of a DFT object: kind 0 flux (E, H), 1 force (offdiag1,
// offdiag2, diag), 2 near2far (F), 3 energy (E, D, H, B)
static dft_chunk *chunk_list(mgb_sim *s, int kind, int handle, int part) {
  if (!s) throw std::runtime_error("null handle");
  auto bad = [] { return std::runtime_error("bad dft object handle or part"); };
  switch (kind) {
    case 0:
      if (handle < 0 || handle >= (int)s->fluxes.size() || part < 0 || part > 1) throw bad();
      return part == 0 ? s->fluxes[handle].E : s->fluxes[handle].H;
    case 1: {
      if (handle < 0 || handle >= (int)s->forces.size() || part < 0 || part > 2) throw bad();
      dft_force &f = s->forces[handle];
      return part == 0 ? f.offdiag1 : part == 1 ? f.offdiag2 : f.diag;
    }
    case 2:
      if (handle < 0 || handle >= (int)s->n2fs.size() || part != 0) throw bad();
      return s->n2fs[handle].F;
    case 3: {
      if (handle < 0 || handle >= (int)s->energies.size() || part < 0 || part > 3) throw bad();
      dft_energy &e = s->energies[handle];
      return part == 0 ? e.E : part == 1 ? e.D : part == 2 ? e.H : e.B;
    }
    default: throw bad();
  }
}

static dft_chunk *flux_part(mgb_sim *s, int handle, int part) { return chunk_list(s, 0, handle, part); }

int mgb_dft_data(mgb_sim *s, int kind, int handle, int part, double *out, size_t *n) {
  try {
    dft_chunk *c = chunk_list(s, kind, handle, part);
    if (!n) throw std::runtime_error("null argument");
    *n = dft_data_size(c);
    if (out) get_dft_data(c, reinterpret_cast<std::complex<double> *>(out), *n);
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_load_dft_data(mgb_sim *s, int kind, int handle, int part, const double *in, size_t n) {
  try {
    if (!in) throw std::runtime_error("null argument");
    load_dft_data(chunk_list(s, kind, handle, part), reinterpret_cast<const std::complex<double> *>(in), n);
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_scale_dft_data(mgb_sim *s, int kind, int handle, int part, double re, double im) {
  try {
    dft_chunk *c = chunk_list(s, kind, handle, part);
    if (c) c->scale_dft(std::complex<double>(re, im));
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_flux_data(mgb_sim *s, int handle, int part, double *out, size_t *n) {
  try {
    dft_chunk *c = flux_part(s, handle, part);
    if (!n) throw std::runtime_error("null argument");
    *n = dft_data_size(c);
    if (out) get_dft_data(c, reinterpret_cast<std::complex<double> *>(out), *n);
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_load_flux_data(mgb_sim *s, int handle, int part, const double *in, size_t n) {
  try {
    if (!in) throw std::runtime_error("null argument");
    load_dft_data(flux_part(s, handle, part), reinterpret_cast<const std::complex<double> *>(in), n);
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_flux_scale(mgb_sim *s, int handle, double re, double im) {
  try {
    if (!s || handle < 0 || handle >= (int)s->fluxes.size()) throw std::runtime_error("bad flux handle");
    s->fluxes[handle].scale_dfts(std::complex<double>(re, im));
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_ldos_create(mgb_sim *s, int nfreq, const double *freqs, int *handle) {
  try {
    if (!s || !freqs || !handle || nfreq < 1) throw std::runtime_error("null argument");
    // the reference's Python layer runs real fields unless a Bloch k makes
    // them complex (fields::use_real_fields in Simulation._init_fields); the
    // LDOS takes the real part of the source current for real fields
    try {
      s->f->use_real_fields();
    } catch (const std::exception &) {
    }
    s->ldoses.emplace_back(new dft_ldos(freqs, (size_t)nfreq));
    *handle = (int)s->ldoses.size() - 1;
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_ldos_update(mgb_sim *s, int handle) {
  try {
    if (!s || handle < 0 || handle >= (int)s->ldoses.size()) throw std::runtime_error("bad ldos handle");
    s->ldoses[handle]->update(*s->f);
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_ldos_results(mgb_sim *s, int handle, double *ldos, double *F, double *J) {
  try {
    if (!s || handle < 0 || handle >= (int)s->ldoses.size()) throw std::runtime_error("bad ldos handle");
    dft_ldos &l = *s->ldoses[handle];
    const size_t nf = l.freq.size();
    if (ldos) {
      double *v = l.ldos();
      std::copy(v, v + nf, ldos);
      delete[] v;
    }
    for (int q = 0; q < 2; q++) {
      double *dst = q == 0 ? F : J;
      if (!dst) continue;
      std::complex<double> *v = q == 0 ? l.F() : l.J();
      for (size_t i = 0; i < nf; i++) {
        dst[2 * i] = v[i].real();
        dst[2 * i + 1] = v[i].imag();
      }
      delete[] v;
    }
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_add_energy(mgb_sim *s, int nreg, const double *regions, int nfreq, const double *freqs, int decimation,
                   int *handle) {
  try {
    if (!s || !regions || !freqs || !handle || nreg < 1) throw std::runtime_error("null argument");
    std::unique_ptr<volume_list> head = region_list(s, nreg, regions);
    s->energies.push_back(s->f->add_dft_energy(head.get(), freqs, (size_t)nfreq, decimation));
    *handle = (int)s->energies.size() - 1;
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_energy(mgb_sim *s, int handle, int which, double *out) {
  try {
    if (!s || !out || handle < 0 || handle >= (int)s->energies.size() || which < 0 || which > 2)
      throw std::runtime_error("bad energy handle");
    dft_energy &e = s->energies[handle];
    double *F = which == 0 ? e.electric() : which == 1 ? e.magnetic() : e.total();
    std::copy(F, F + e.freq.size(), out);
    delete[] F;
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_add_force(mgb_sim *s, int nreg, const double *regions, int nfreq, const double *freqs, int decimation,
                  int *handle) {
  try {
    if (!s || !regions || !freqs || !handle || nreg < 1) throw std::runtime_error("null argument");
    std::unique_ptr<volume_list> head = region_list(s, nreg, regions);
    s->forces.push_back(s->f->add_dft_force(head.get(), freqs, (size_t)nfreq, decimation));
    *handle = (int)s->forces.size() - 1;
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_force(mgb_sim *s, int handle, double *out) {
  try {
    if (!s || !out || handle < 0 || handle >= (int)s->forces.size()) throw std::runtime_error("bad force handle");
    double *F = s->forces[handle].force();
    std::copy(F, F + s->forces[handle].freq.size(), out);
    delete[] F;
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

static dft_near2far &n2f_of(mgb_sim *s, int handle) {
  if (!s || handle < 0 || handle >= (int)s->n2fs.size()) throw std::runtime_error("bad near2far handle");
  return s->n2fs[handle];
}

static vec point_of(int dim, const double *p) {
  if (dim == 1) return vec(p[2]);
  if (dim == 2) return vec(p[0], p[1]);
  return vec(p[0], p[1], p[2]);
}

int mgb_add_near2far(mgb_sim *s, int nreg, const double *regions, int nfreq, const double *freqs, int decimation,
                     int nperiods, int *handle) {
  try {
    if (!s || !regions || !freqs || !handle || nreg < 1) throw std::runtime_error("null argument");
    std::unique_ptr<volume_list> head = region_list(s, nreg, regions);
    s->n2fs.push_back(s->f->add_dft_near2far(head.get(), freqs, (size_t)nfreq, decimation, nperiods));
    *handle = (int)s->n2fs.size() - 1;
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_near2far_points(mgb_sim *s, int handle, int npts, const double *xyz, double *out) {
  try {
    dft_near2far &n = n2f_of(s, handle);
    if (npts < 0 || (npts > 0 && (!xyz || !out))) throw std::runtime_error("null argument");
    std::vector<vec> pts;
    for (int i = 0; i < npts; i++)
      pts.push_back(point_of(s->dim, xyz + 3 * i));
    n.farfields_at(pts, reinterpret_cast<std::complex<double> *>(out));
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_near2far_array(mgb_sim *s, int handle, const double center[3], const double size[3], double resolution,
                       double *out, int dims[3], int *rank) {
  try {
    dft_near2far &n = n2f_of(s, handle);
    if (!center || !size || !dims || !rank) throw std::runtime_error("null argument");
    const volume v = mkvol(s->dim, center, size);
    int r = 0;
    size_t dd[3] = {1, 1, 1}, N = 1;
    if (!out) {
      // the grid only (get_farfields_array's sizing, no evaluation)
      LOOP_OVER_DIRECTIONS(v.dim, q) {
        size_t k = (size_t)int(std::floor(v.in_direction(q) * resolution));
        dd[r++] = k <= 1 ? 1 : k;
      }
    }
    else {
      double *EH = n.get_farfields_array(v, r, dd, N, resolution);
      if (EH) {
        std::copy(EH, EH + 12 * N * n.freq.size(), out);
        delete[] EH;
      }
      // get_farfields_array collapsed singleton directions; report the grid
      r = 0;
      dd[0] = dd[1] = dd[2] = 1;
      LOOP_OVER_DIRECTIONS(v.dim, q) {
        size_t k = (size_t)int(std::floor(v.in_direction(q) * resolution));
        dd[r++] = k <= 1 ? 1 : k;
      }
    }
    for (int q = 0; q < 3; q++)
      dims[q] = (int)dd[q];
    *rank = r;
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_near2far_flux(mgb_sim *s, int handle, int direction, const double center[3], const double size[3],
                      double resolution, double *out) {
  try {
    dft_near2far &n = n2f_of(s, handle);
    if (!center || !size || !out || direction < 0 || direction > 2) throw std::runtime_error("bad argument");
    double *F = n.flux(meep::direction(direction), mkvol(s->dim, center, size), resolution);
    std::copy(F, F + n.freq.size(), out);
    delete[] F;
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_near2far_scale(mgb_sim *s, int handle, double re, double im) {
  try {
    n2f_of(s, handle).scale_dfts(std::complex<double>(re, im));
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_near2far_medium(mgb_sim *s, int handle, double *eps, double *mu) {
  try {
    dft_near2far &n = n2f_of(s, handle);
    if (eps) *eps = n.eps;
    if (mu) *mu = n.mu;
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_add_dft_fields(mgb_sim *s, int ncomp, const int *components, const double center[3],
                       const double size[3], int nfreq, const double *freqs, int yee_grid, int decimation,
                       int *handle) {
  try {
    if (!s || !components || !freqs || !handle) throw std::runtime_error("null argument");
    std::vector<component> cs;
    for (int q = 0; q < ncomp; q++)
      cs.push_back((component)components[q]);
    s->dfts.push_back(s->f->add_dft_fields(cs.data(), ncomp, mkvol(s->dim, center, size), freqs, (size_t)nfreq,
                                           yee_grid == 0, decimation));
    *handle = (int)s->dfts.size() - 1;
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_dft_fields_array(mgb_sim *s, int handle, int component_, int ifreq, double *out, int shape[3]) {
  try {
    if (!s || !shape || handle < 0 || handle >= (int)s->dfts.size()) throw std::runtime_error("bad handle");
    const dft_fields &D = s->dfts[handle];
    if (ifreq < 0 || ifreq >= (int)D.freq.size()) throw std::runtime_error("frequency index out of range");
    for (dft_chunk *ch = D.chunks; ch; ch = ch->next_in_dft) {
      if ((int)ch->c != component_) continue;
      size_t np = 1;
      int k = 0;
      for (int d = 0; d < 3; d++) {
        if ((s->dim == 1 && d != 2) || (s->dim == 2 && d == 2)) {
          shape[d] = 1;
          continue;
        }
        shape[d] = (ch->ie.in_direction((direction)d) - ch->is.in_direction((direction)d)) / 2 + 1;
        np *= (size_t)shape[d];
        k++;
      }
      (void)k;
      if (np != ch->N) throw std::runtime_error("internal: dft chunk size mismatch");
      if (out) {
        sync_dfts(*s->f);
        const size_t nf = D.freq.size();
        for (size_t i = 0; i < np; i++) {
          out[2 * i] = std::real(ch->dft[i * nf + ifreq]);
          out[2 * i + 1] = std::imag(ch->dft[i * nf + ifreq]);
        }
      }
      return 0;
    }
    throw std::runtime_error("meep: component not in this DFT object");
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_step(mgb_sim *s, int n) {
  try {
    if (!s) throw std::runtime_error("null simulation");
    if (n > 0) step_n(*s->f, n);
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_time(const mgb_sim *s, double *time, double *round_time, double *dt, int *t) {
  if (!s) return -1;
  if (time) *time = s->f->time();
  if (round_time) *round_time = s->f->round_time();
  if (dt) *dt = s->f->dt;
  if (t) *t = s->f->t;
  return 0;
}

int mgb_get_field_points(mgb_sim *s, int component_, int n, const double *xyz, double *re, double *im) {
  try {
    if (!s || !xyz || !re) throw std::runtime_error("null argument");
    for (int q = 0; q < n; q++) {
      const std::complex<double> v = s->f->get_field((component)component_, mkvec(s->dim, xyz + 3 * q));
      re[q] = v.real();
      if (im) im[q] = v.imag();
    }
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_add_material_grid(mgb_sim *s, const double center[3], const double size[3], const int n[3],
                          const double *weights, double beta, double eta, const double eps1[3],
                          const double eps2[3]) {
  try {
    if (!s || !center || !size || !n || !weights || !eps1 || !eps2) throw std::runtime_error("null argument");
    s->s->add_material_grid(center, size, n, weights, beta, eta, eps1, eps2);
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_use_bloch(mgb_sim *s, const double k[3]) {
  try {
    if (!s || !k) throw std::runtime_error("null argument");
    s->f->use_bloch(mkvec(s->dim, k));
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_yee_array(mgb_sim *s, int component_, int part, double *out, long long *n) {
  try {
    if (!s || !n) throw std::runtime_error("null argument");
    const grid_volume &gv = s->f->gv;
    const component c = (component)component_;
    int cnt[3] = {1, 1, 1};
    direction ds[3] = {X, Y, Z};
    int nd = 0;
    LOOP_OVER_DIRECTIONS(gv.dim, d) {
      ds[nd] = d;
      cnt[nd] = gv.num_direction(d) + 1;
      nd++;
    }
    *n = (long long)cnt[0] * cnt[1] * cnt[2];
    if (!out) return 0;
    const ivec base = gv.little_corner() + gv.iyee_shift(c);
    long long q = 0;
    for (int a = 0; a < cnt[0]; a++)
      for (int b = 0; b < cnt[1]; b++)
        for (int e = 0; e < cnt[2]; e++) {
          ivec p = base;
          const int k[3] = {a, b, e};
          for (int r = 0; r < nd; r++)
            p.set_direction(ds[r], p.in_direction(ds[r]) + 2 * k[r]);
          const std::complex<double> v = s->f->get_field(c, p, false);
          out[q++] = part ? v.imag() : v.real();
        }
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int mgb_get_epsilon_points(mgb_sim *s, int n, const double *xyz, double *eps) {
  try {
    if (!s || !xyz || !eps) throw std::runtime_error("null argument");
    for (int q = 0; q < n; q++)
      eps[q] = s->geo.at(mkvec(s->dim, xyz + 3 * q)).eps[0];
    return 0;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

} // extern "C"
