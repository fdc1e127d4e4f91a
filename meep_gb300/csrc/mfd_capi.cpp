// C ABI of the stepping engine (declared in include/mfd.h).  Owns the Plan
// and the backend; every entry point converts exceptions to a status code and
// a last-error string, the way the reference's SWIG layer maps meep::abort to
// a Python exception (python/meep.i:1365-1380).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>

#include "mfd.h"
#include "mfd_backend.hpp"

using namespace mfd;

struct mfd_sim {
  std::unique_ptr<Plan> plan;
  std::unique_ptr<Backend> be;
  bool setup_done = false;
  int64_t t = 0;
  // differentiation state
  bool design = false;
  int64_t design_points = 0;

  int64_t fwd_t0 = -1, fwd_n = 0;
  int fwd_K = 0;
  std::vector<int> snaps;
};

static thread_local std::string g_last_error;

#define MFD_TRY try {
#define MFD_CATCH                                                                                  \
  }                                                                                                \
  catch (const std::exception &e) {                                                                \
    g_last_error = e.what();                                                                       \
    return -1;                                                                                     \
  }                                                                                                \
  catch (...) {                                                                                    \
    g_last_error = "meep: unknown error";                                                          \
    return -1;                                                                                     \
  }                                                                                                \
  return 0;

static void need(bool ok, const char *msg) {
  if (!ok) throw Error(msg);
}

static void check_comp(mfd_sim *s, int c) {
  need(s && s->plan, "null simulation handle");
  need(c >= 0 && c < NC, "component out of range");
}

extern "C" {

const char *mfd_last_error(void) { return g_last_error.c_str(); }

int mfd_create(const mfd_grid *grid, mfd_sim **out) {
  MFD_TRY
  need(grid && out, "null argument to mfd_create");
  *out = nullptr;
  auto s = std::unique_ptr<mfd_sim>(new mfd_sim);
  s->plan.reset(new Plan(*grid));
  s->be.reset(make_backend(*s->plan));
  *out = s.release();
  MFD_CATCH
}

void mfd_destroy(mfd_sim *sim) { delete sim; }

int mfd_set_chi1inv(mfd_sim *s, int c, int d, const double *values) {
  MFD_TRY
  check_comp(s, c);
  need(d >= 0 && d < 3, "direction out of range");
  need(ctype(c) == MFD_E || ctype(c) == MFD_H, "chi1inv is defined for E and H components");
  need(!s->setup_done, "materials must be set before the first step");
  need(values != nullptr, "null array");
  s->plan->chi1inv[c][d].assign(values, values + s->plan->ndense);
  MFD_CATCH
}

int mfd_set_conductivity(mfd_sim *s, int c, const double *values) {
  MFD_TRY
  check_comp(s, c);
  need(ctype(c) == MFD_D || ctype(c) == MFD_B, "conductivity is stored on D or B components");
  need(!s->setup_done, "materials must be set before the first step");
  need(values != nullptr, "null array");
  Plan &p = *s->plan;
  p.cond[c].assign(values, values + p.ndense);
  bool any = false;
  for (double v : p.cond[c])
    any = any || v != 0.0;
  if (!any) p.cond[c].clear(); // trivial: dropped, as the reference does
  p.compute_cond_chunks(c);
  MFD_CATCH
}

int mfd_add_lorentzian(mfd_sim *s, int ft, double omega0, double gamma, int drude,
                       const double *const sigma[3]) {
  MFD_TRY
  need(s && s->plan, "null simulation handle");
  need(ft == MFD_E, "only electric susceptibilities are supported");
  need(!s->setup_done, "susceptibilities must be added before the first step");
  need((int)s->plan->poles.size() < MAX_POLES, "too many susceptibility poles");
  Pole pole;
  pole.ft = ft;
  pole.omega0 = omega0;
  pole.gamma = gamma;
  pole.drude = drude != 0;
  for (int d = 0; d < 3; d++)
    if (sigma && sigma[d]) {
      pole.sigma[d].assign(sigma[d], sigma[d] + s->plan->ndense);
      bool any = false;
      for (double v : pole.sigma[d])
        any = any || v != 0.0;
      if (!any) pole.sigma[d].clear();
    }
  // the reference prepends each new susceptibility (src/anisotropic_averaging.cpp:414-416)
  s->plan->poles.insert(s->plan->poles.begin(), pole);
  MFD_CATCH
}

int mfd_add_gaussian_src(mfd_sim *s, double freq, double fwidth_or_width, double start,
                         double end, int explicit_window, int is_integrated, int *id) {
  MFD_TRY
  need(s && s->plan && id, "null argument");
  SrcTime st = explicit_window ? SrcTime::gaussian_window(freq, fwidth_or_width, start, end)
                               : SrcTime::gaussian(freq, fwidth_or_width, start > 0 ? start : 5.0);
  st.integrated = is_integrated != 0;
  s->plan->srcs.push_back(st);
  *id = (int)s->plan->srcs.size() - 1;
  MFD_CATCH
}

int mfd_add_continuous_src(mfd_sim *s, double fre, double fim, double width, double start,
                           double end, double slowness, int is_integrated, int *id) {
  MFD_TRY
  need(s && s->plan && id, "null argument");
  SrcTime st = SrcTime::continuous({fre, fim}, width, start, end, slowness);
  st.integrated = is_integrated != 0;
  s->plan->srcs.push_back(st);
  *id = (int)s->plan->srcs.size() - 1;
  MFD_CATCH
}

int mfd_add_source_points(mfd_sim *s, int c, int src_id, size_t npts, const int64_t *idx,
                          const double *amp) {
  MFD_TRY
  check_comp(s, c);
  Plan &p = *s->plan;
  need(ctype(c) == MFD_E || ctype(c) == MFD_H, "sources are given on E or H components");
  need(p.have[c], "source component is not allocated");
  need(src_id >= 0 && src_id < (int)p.srcs.size(), "unknown source time id");
  need(!s->setup_done, "sources must be added before the first step");
  if (ctype(c) == MFD_H && p.srcs[src_id].integrated)
    throw Error("integrated magnetic sources are not supported; set is_integrated = false");
  SourceGroup gsrc;
  gsrc.c = c;
  gsrc.src = src_id;
  for (size_t j = 0; j < npts; j++) {
    need(idx[j] >= 0 && idx[j] < p.ndense, "source index out of range");
    gsrc.idx.push_back(idx[j]);
    gsrc.amp.emplace_back(amp[2 * j], amp[2 * j + 1]);
  }
  if (!gsrc.idx.empty()) p.sources.push_back(std::move(gsrc));
  MFD_CATCH
}

int mfd_add_dft(mfd_sim *s, int c, const int lo[3], const int hi[3], const double *const w[3],
                double dV, int include_weights, double scale_re, double scale_im, int centered,
                size_t nfreq, const double *freq, int decimation, int *id) {
  MFD_TRY
  check_comp(s, c);
  Plan &p = *s->plan;
  need(p.have[c], "DFT component is not allocated");
  need(nfreq > 0 && freq, "DFT needs at least one frequency");
  need(decimation >= 1, "decimation factor must be >= 1");
  need(id != nullptr, "null id");
  Monitor m;
  m.c = c;
  m.npts = 1;
  for (int d = 0; d < 3; d++) {
    m.lo[d] = lo[d];
    m.hi[d] = hi[d];
    need(lo[d] <= hi[d] && lo[d] >= 0 && hi[d] < p.ext[d], "DFT box out of range");
    if (centered && p.present[d] && p.shift[c][d] == 0)
      need(hi[d] + 1 < p.ext[d], "centred DFT box needs a neighbour point");
    int n = hi[d] - lo[d] + 1;
    m.npts *= n;
    if (p.present[d]) {
      need(w && w[d], "missing DFT weights");
      m.w[d].assign(w[d], w[d] + n);
    }
  }
  m.dV = dV;
  need(include_weights >= 0 && include_weights <= 2, "include_weights must be 0, 1 or 2");
  m.include_weights = include_weights != 0;
  m.sqrt_weights = include_weights == 2;
  m.scale = {scale_re, scale_im};
  m.centered = centered != 0;
  m.freq.assign(freq, freq + nfreq);
  m.decimation = decimation;
  p.monitors.push_back(m);
  *id = (int)p.monitors.size() - 1;
  if (s->setup_done) s->be->add_monitor(p, *id);
  MFD_CATCH
}

static void ensure_setup(mfd_sim *s) {
  Plan &p = *s->plan;
  if (!s->setup_done) {
    s->be->setup(p);
    for (int i = 0; i < (int)p.monitors.size(); i++)
      s->be->add_monitor(p, i);
    s->setup_done = true;
  }
}

// calc_sources at t, t+dt/2 and t+dt (src/step.cpp:64-108)
static void source_values(Plan &p, int64_t t, std::vector<SrcStepValues> &vals) {
  vals.resize(p.srcs.size());
  double time = t * p.dt;
  for (size_t k = 0; k < p.srcs.size(); k++) {
    SrcTime &st = p.srcs[k];
    st.update(time, p.dt);
    vals[k].cur_b = st.cur_current;
    st.update(time + 0.5 * p.dt, p.dt);
    vals[k].cur_d = st.cur_current;
    st.update(time + p.dt, p.dt);
    vals[k].dip_e = st.cur_dipole;
  }
}

int mfd_step(mfd_sim *s, int n) {
  MFD_TRY
  need(s && s->plan, "null simulation handle");
  Plan &p = *s->plan;
  ensure_setup(s);
  std::vector<SrcStepValues> vals;
  s->be->begin_steps();
  for (int it = 0; it < n; it++) {
    source_values(p, s->t, vals);
    s->be->step(p, s->t, vals);
    s->t += 1;
  }
  s->be->end_steps();
  MFD_CATCH
}

int mfd_design(mfd_sim *s, int ncomp, const int *comps, const int lo[3], const int hi[3]) {
  MFD_TRY
  need(s && s->plan && comps && lo && hi, "null argument");
  need(ncomp >= 1 && ncomp <= 3, "1 to 3 design components");
  ensure_setup(s);
  s->be->set_design(*s->plan, std::vector<int>(comps, comps + ncomp), lo, hi);
  s->design = true;
  s->design_points = (int64_t)ncomp * (hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1);
  MFD_CATCH
}

int mfd_add_material_grid(mfd_sim *s, const double center[3], const double size[3], const int n[3],
                          const double *weights, double beta, double eta, const double eps1[3],
                          const double eps2[3], int *id) {
  MFD_TRY
  need(s && s->plan && center && size && n && weights && eps1 && eps2, "null argument");
  need(!s->setup_done, "materials must be set before the first step");
  need(n[0] >= 1 && n[1] >= 1 && n[2] >= 1, "material grid sizes must be at least 1");
  need(beta >= 0 && eta >= 0 && eta <= 1, "material grid projection needs beta >= 0 and eta in [0, 1]");
  Plan::MatGrid mg;
  for (int d = 0; d < 3; d++) {
    need(size[d] >= 0 && std::isfinite(size[d]) && std::isfinite(center[d]) &&
             std::fabs(center[d]) + 0.5 * size[d] < 1e6, "invalid material grid block");
    need(eps1[d] > 0 && eps2[d] > 0, "material grid permittivities must be positive");
    mg.spec.center[d] = center[d];
    mg.spec.size[d] = size[d];
    mg.spec.n[d] = n[d];
    mg.spec.eps1[d] = eps1[d];
    mg.spec.eps2[d] = eps2[d];
  }
  mg.spec.beta = beta;
  mg.spec.eta = eta;
  mg.u.assign(weights, weights + (size_t)n[0] * n[1] * n[2]);
  for (double w : mg.u)
    need(w >= 0.0 && w <= 1.0, "The weights parameter of MaterialGrid must be in the range [0,1].");
  s->plan->matgrids.push_back(std::move(mg));
  if (id) *id = int(s->plan->matgrids.size()) - 1;
  MFD_CATCH
}

int mfd_material_grid_vjp(mfd_sim *s, int id, int ncomp, const int *comps, const int lo[3], const int hi[3],
                          const double *grad_chi1inv, double *grad_weights) {
  MFD_TRY
  need(s && s->plan && comps && lo && hi && grad_chi1inv && grad_weights, "null argument");
  need(id >= 0 && id < int(s->plan->matgrids.size()), "material grid id out of range");
  need(ncomp >= 1 && ncomp <= 3, "1 to 3 components");
  const Plan &p = *s->plan;
  for (int q = 0; q < ncomp; q++)
    need(comps[q] >= 0 && comps[q] < 3 && p.have[comps[q]], "components must be allocated E components");
  for (int d = 0; d < 3; d++)
    need(lo[d] >= 0 && lo[d] <= hi[d] && hi[d] <= (p.present[d] ? p.N[d] : 0), "box out of range");
  ensure_setup(s);
  s->be->matgrid_vjp(*s->plan, id, std::vector<int>(comps, comps + ncomp), lo, hi, grad_chi1inv, grad_weights);
  MFD_CATCH
}

int mfd_forward(mfd_sim *s, int n, int K) {
  MFD_TRY
  need(s && s->plan, "null simulation handle");
  need(s->design, "call mfd_design before mfd_forward");
  need(!s->plan->complex_fields, "the adjoint does not support complex (Bloch) fields");
  need(n >= 1 && K >= -1, "invalid step counts");
  Plan &p = *s->plan;
  ensure_setup(s);
  if (K < 0) {
    // automatic: record the design-point D of every step when that fits the
    // budget (no recomputation), else checkpoints every ceil(sqrt(n)) steps
    double budget = 16e9;
    if (const char *e = getenv("MFD_RECORD_BUDGET_GB")) budget = atof(e) * 1e9;
    double need_bytes = (double)s->design_points * n * (p.g.precision / 8);
    K = need_bytes <= budget ? 0 : (int)std::ceil(std::sqrt((double)n));
  }
  s->fwd_t0 = s->t;
  s->fwd_n = n;
  s->fwd_K = K;
  s->snaps.clear();
  if (K == 0) s->be->alloc_record(p, n);
  std::vector<SrcStepValues> vals;
  s->be->begin_steps();
  for (int it = 0; it < n; it++) {
    if (K > 0 && it % K == 0) s->snaps.push_back(s->be->snapshot(p));
    source_values(p, s->t, vals);
    s->be->step(p, s->t, vals);
    if (K == 0) s->be->record_design(p, it);
    s->t += 1;
  }
  s->be->end_steps();
  MFD_CATCH
}

int mfd_backward(mfd_sim *s, int nmon, const int *ids, const double *const *grads, double *grad_out) {
  MFD_TRY
  need(s && s->plan && grad_out, "null argument");
  need(s->fwd_t0 >= 0, "call mfd_forward before mfd_backward");
  need(nmon >= 0 && (nmon == 0 || (ids && grads)), "invalid monitor gradients");
  Plan &p = *s->plan;
  for (int q = 0; q < nmon; q++) {
    need(ids[q] >= 0 && ids[q] < (int)p.monitors.size(), "unknown monitor id");
    need(!p.monitors[ids[q]].sqrt_weights, "monitors with square-root weights (force) have no adjoint here");
  }
  Backend &be = *s->be;
  be.begin_steps();
  be.adjoint_begin(p, nmon, ids, grads);
  const int64_t t0 = s->fwd_t0, n = s->fwd_n;
  if (s->fwd_K == 0) {
    for (int64_t st = t0 + n - 1; st >= t0; st--)
      be.adjoint_step(p, st, st - t0);
  }
  else {
    const int K = s->fwd_K;
    be.alloc_record(p, K);
    std::vector<SrcStepValues> vals;
    for (int seg = (int)s->snaps.size() - 1; seg >= 0; seg--) {
      const int64_t a = t0 + (int64_t)seg * K;
      const int64_t len = std::min<int64_t>(K, t0 + n - a);
      be.restore(p, s->snaps[seg]);
      be.set_skip_dft(true);
      for (int64_t it = 0; it < len; it++) {
        source_values(p, a + it, vals);
        be.step(p, a + it, vals);
        be.record_design(p, it);
      }
      be.set_skip_dft(false);
      for (int64_t st = a + len - 1; st >= a; st--)
        be.adjoint_step(p, st, st - a);
    }
  }
  be.adjoint_end(p, grad_out);
  be.end_steps();
  s->fwd_t0 = -1;
  MFD_CATCH
}

int mfd_get_time(const mfd_sim *s, int64_t *t, double *dt) {
  MFD_TRY
  need(s && s->plan, "null simulation handle");
  if (t) *t = s->t;
  if (dt) *dt = s->plan->dt;
  MFD_CATCH
}

int mfd_get_field(mfd_sim *s, int c, double *out) {
  MFD_TRY
  check_comp(s, c);
  need(out != nullptr, "null output");
  Plan &p = *s->plan;
  if (!p.have[c]) {
    std::memset(out, 0, sizeof(double) * p.ndense);
    return 0;
  }
  if (!s->setup_done) {
    s->be->setup(p);
    for (int i = 0; i < (int)p.monitors.size(); i++)
      s->be->add_monitor(p, i);
    s->setup_done = true;
  }
  s->be->get_field(p, c, out);
  MFD_CATCH
}

int mfd_get_field_im(mfd_sim *s, int c, double *out) {
  MFD_TRY
  check_comp(s, c);
  need(out != nullptr, "null output");
  Plan &p = *s->plan;
  if (!p.have[c] || !p.complex_fields) {
    std::memset(out, 0, sizeof(double) * p.ndense);
    return 0;
  }
  ensure_setup(s);
  s->be->get_field_im(p, c, out);
  MFD_CATCH
}

int mfd_subpixel_rows(int dim, int cdir, int64_t npix, const double *lo, const double *hi, double tol, int maxeval,
                      int nobj, const mfd_object *objs, double eps_default, double *rows) {
  MFD_TRY
  need(dim >= 1 && dim <= 3, "dim must be 1, 2 or 3");
  need(cdir >= 0 && cdir < 3, "cdir must be 0, 1 or 2");
  need(npix >= 0, "negative pixel count");
  need(nobj >= 0 && (nobj == 0 || objs), "null object list");
  need(npix == 0 || (lo && hi && rows), "null pixel or row array");
  need(maxeval >= 0, "negative maxeval");
  for (int q = 0; q < nobj; q++)
    need(objs[q].kind >= 0 && objs[q].kind <= 2, "unknown object kind");
  if (npix > 0) subpixel_rows(dim, cdir, npix, lo, hi, tol, maxeval, nobj, objs, eps_default, rows);
  return 0;
  MFD_CATCH
}

int mfd_set_bloch(mfd_sim *s, const int periodic[3], const double k[3]) {
  MFD_TRY
  need(s && s->plan && periodic && k, "null argument");
  need(!s->setup_done, "boundaries must be set before the first step");
  s->plan->set_bloch(periodic, k);
  MFD_CATCH
}

int mfd_get_dft(mfd_sim *s, int id, double *out, size_t *npts, size_t *nfreq) {
  MFD_TRY
  need(s && s->plan, "null simulation handle");
  Plan &p = *s->plan;
  need(id >= 0 && id < (int)p.monitors.size(), "unknown monitor id");
  if (npts) *npts = p.monitors[id].npts;
  if (nfreq) *nfreq = p.monitors[id].freq.size();
  if (out) {
    if (!s->setup_done) {
      size_t n = p.monitors[id].npts * p.monitors[id].freq.size() * 2;
      std::memset(out, 0, n * sizeof(double));
    }
    else
      s->be->get_dft(p, id, out);
  }
  MFD_CATCH
}

int mfd_flux(mfd_sim *s, int npairs, const int *idE, const int *idH, double *out) {
  MFD_TRY
  need(s && s->plan && out, "null argument");
  Plan &p = *s->plan;
  need(npairs >= 1, "flux needs at least one monitor pair");
  size_t nf = p.monitors[idE[0]].freq.size();
  for (int k = 0; k < npairs; k++) {
    need(idE[k] >= 0 && idE[k] < (int)p.monitors.size() && idH[k] >= 0 &&
             idH[k] < (int)p.monitors.size(),
         "unknown monitor id");
    need(p.monitors[idE[k]].npts == p.monitors[idH[k]].npts, "paired monitors differ in size");
    need(p.monitors[idE[k]].freq.size() == nf && p.monitors[idH[k]].freq.size() == nf,
         "paired monitors differ in frequencies");
  }
  if (!s->setup_done) {
    for (size_t i = 0; i < nf; i++)
      out[i] = 0.0;
    return 0;
  }
  s->be->flux(p, npairs, idE, idH, out);
  MFD_CATCH
}

int mfd_src_current(const mfd_sim *s, int src_id, double time, double *out) {
  MFD_TRY
  need(s && s->plan && out, "null argument");
  const Plan &p = *s->plan;
  need(src_id >= 0 && src_id < (int)p.srcs.size(), "unknown source id");
  const std::complex<double> c = p.srcs[src_id].current(time, p.dt);
  out[0] = c.real();
  out[1] = c.imag();
  MFD_CATCH
}

int mfd_scale_dft(mfd_sim *s, int id, double s_re, double s_im) {
  MFD_TRY
  need(s && s->plan, "null simulation handle");
  Plan &p = *s->plan;
  need(id >= 0 && id < (int)p.monitors.size(), "unknown monitor id");
  if (s->setup_done) s->be->scale_dft(p, id, {s_re, s_im});
  MFD_CATCH
}

int mfd_set_dft(mfd_sim *s, int id, const double *in) {
  MFD_TRY
  need(s && s->plan && in, "null argument");
  Plan &p = *s->plan;
  need(id >= 0 && id < (int)p.monitors.size(), "unknown monitor id");
  // the sums live in the backend once it is set up: set it up now (the
  // reference loads flux data before the run, after the sources and monitors)
  ensure_setup(s);
  s->be->set_dft(p, id, in);
  MFD_CATCH
}

int mfd_farfield(mfd_sim *s, int nsheet, const int *ids, const int *src_comp, const double *is_half,
                 const double *rshift, double eps, double mu, const int periodic_dir[2], const int periodic_n[2],
                 const double periodic_k[2], const double period[2], int64_t nx, const double *x, double *out) {
  MFD_TRY
  need(s && s->plan, "null simulation handle");
  Plan &p = *s->plan;
  need(nsheet >= 1 && ids && src_comp && is_half && rshift, "near2far needs at least one monitor");
  need(nx >= 0 && (nx == 0 || (x && out)), "null far-point or output array");
  need(periodic_dir && periodic_n && periodic_k && period, "null periodicity argument");
  N2FSpec sp{};
  if (p.present[0] && p.present[1] && p.present[2]) sp.dim = 3;
  else if (p.present[0] && p.present[1] && !p.present[2]) sp.dim = 2;
  else throw Error("meep: only 2d or 3d far-field computation is supported");
  need(eps > 0 && mu > 0, "near2far medium must have eps > 0 and mu > 0");
  sp.eps = eps;
  sp.mu = mu;
  sp.inva = p.inva;
  for (int j = 0; j < 2; j++) {
    need(periodic_dir[j] >= -1 && periodic_dir[j] < 3, "periodic direction out of range");
    need(periodic_n[j] >= 0 && (periodic_dir[j] >= 0 || periodic_n[j] == 0), "bad periodic image count");
    sp.pdir[j] = periodic_dir[j];
    sp.pn[j] = periodic_n[j];
    sp.pk[j] = periodic_k[j];
    sp.period[j] = period[j];
  }
  std::vector<N2FSheet> sh(nsheet);
  size_t nf = 0;
  for (int i = 0; i < nsheet; i++) {
    need(ids[i] >= 0 && ids[i] < (int)p.monitors.size(), "unknown monitor id");
    need(src_comp[i] >= 0 && src_comp[i] < 6, "equivalent source must be an E or H component");
    const Monitor &m = p.monitors[ids[i]];
    need(!m.centered, "near2far monitors must be on the Yee grid (centered = 0)");
    if (i == 0) nf = m.freq.size();
    need(m.freq.size() == nf, "near2far monitors differ in frequencies");
    sh[i].id = ids[i];
    sh[i].c0 = src_comp[i];
    for (int d = 0; d < 3; d++) {
      sh[i].is_half[d] = is_half[3 * i + d];
      sh[i].rshift[d] = rshift[3 * i + d];
    }
  }
  if (nx == 0) return 0;
  if (!s->setup_done) {
    std::memset(out, 0, sizeof(double) * 12 * nf * (size_t)nx);
    return 0;
  }
  s->be->farfield(p, sp, sh, nx, x, out);
  MFD_CATCH
}

int mfd_green(int dim, int c0, double freq, double eps, double mu, double f0_re, double f0_im, int64_t n,
              const double *x, const double *x0, double *out) {
  MFD_TRY
  need(dim == 2 || dim == 3, "wrong dimensionality in green's function (2 or 3)");
  need(c0 >= 0 && c0 < 6, "unrecognized source type");
  need(n >= 0 && (n == 0 || (x && x0 && out)), "null point array");
  if (n > 0) green_eval(dim, c0, freq, eps, mu, f0_re, f0_im, n, x, x0, out);
  MFD_CATCH
}

int64_t mfd_kernel_launches(const mfd_sim *s) { return s && s->be ? s->be->launches() : 0; }

double mfd_last_step_ms(const mfd_sim *s) { return s && s->be ? s->be->last_step_ms() : 0.0; }

} // extern "C"
