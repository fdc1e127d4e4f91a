// Plan construction: grid layout, PML coefficient tables, curl plan and the
// source time functions.  See mfd_plan.hpp for the model.
#include "mfd_plan.hpp"

#include <utility>

#include <cmath>
#include <cstring>
#include <algorithm>

namespace mfd {

static const double pi = 3.141592653589793238462643383276;

// ------------------------------------------------------------ source times

// Bandwidth of the Gaussian at 1e-7 below its peak (src/sources.cpp:67-70).
static double gaussian_bandwidth(double width) {
  double tol = 1e-7;
  return std::sqrt(-2.0 * std::log(tol)) / (width * pi);
}

// gaussian_src_time(f, fwidth, s) (src/sources.cpp:72-84)
SrcTime SrcTime::gaussian(double f, double fw, double s) {
  SrcTime st;
  st.kind = 0;
  st.freq = f;
  st.width = 1.0 / fw;
  st.peak_time = st.width * s;
  st.cutoff = st.width * s;
  st.fwidth = gaussian_bandwidth(st.width);
  while (std::exp(-st.cutoff * st.cutoff / (2 * st.width * st.width)) < 1e-100)
    st.cutoff *= 0.9;
  st.cutoff = float(st.cutoff);
  return st;
}

// gaussian_src_time(f, w, start, end) (src/sources.cpp:86-96)
SrcTime SrcTime::gaussian_window(double f, double w, double st_, double et) {
  SrcTime st;
  st.kind = 0;
  st.freq = f;
  st.width = w;
  st.peak_time = 0.5 * (st_ + et);
  st.cutoff = (et - st_) * 0.5;
  st.fwidth = gaussian_bandwidth(st.width);
  while (std::exp(-st.cutoff * st.cutoff / (2 * st.width * st.width)) < 1e-100)
    st.cutoff *= 0.9;
  st.cutoff = float(st.cutoff);
  return st;
}

SrcTime SrcTime::continuous(std::complex<double> f, double w, double st_, double et, double s) {
  SrcTime st;
  st.kind = 1;
  st.cfreq = f;
  st.width = w;
  st.start = float(st_);
  st.end = float(et);
  st.slowness = s;
  return st;
}

// dipole moments: gaussian_src_time::dipole (src/sources.cpp:98-110),
// continuous_src_time::dipole (src/sources.cpp:128-146).  The arithmetic is the
// reference's formula, evaluated with std::complex<double>.
std::complex<double> SrcTime::dipole(double time) const {
  using cd = std::complex<double>;
  if (kind == 0) {
    double tt = time - peak_time;
    if (float(std::fabs(tt)) > cutoff) return 0.0;
    cd amp = 1.0 / cd(0, -2 * pi * freq);
    return std::exp(-tt * tt / (2 * width * width)) * std::polar(1.0, -2 * pi * freq * tt) * amp;
  }
  float rtime = float(time);
  if (rtime < start || rtime > end) return 0.0;
  cd amp = 1.0 / (cd(0, -1.0) * (2 * pi) * cfreq);
  if (width == 0.0) return std::exp(cd(0, -1.0) * (2 * pi) * cfreq * time) * amp;
  double ts = (time - start) / width - slowness;
  double te = (end - time) / width - slowness;
  return std::exp(cd(0, -1.0) * (2 * pi) * cfreq * time) * amp * (1.0 + std::tanh(ts)) *
         (1.0 + std::tanh(te)) * 0.25;
}

// ------------------------------------------------------------------- plan

// Distance into the PML, quantised to half pixels (src/structure.cpp:622-625).
static inline double pml_x(int i, double dx, double bloc, double a) {
  double here = i * 0.5 / a;
  return (0.5 / a * ((int)(dx * (2 * a) + 0.5) - (int)(std::fabs(bloc - here) * (2 * a) + 0.5)));
}

Plan::Plan(const mfd_grid &grid) : g(grid) {
  if (g.dim < 1 || g.dim > 3) throw Error("dim must be 1, 2 or 3");
  if (g.a <= 0) throw Error("resolution must be positive");
  if (g.precision != 32 && g.precision != 64) throw Error("precision must be 32 or 64");
  if (g.dim == 1) present[2] = true;
  if (g.dim >= 2) present[0] = present[1] = true;
  if (g.dim == 3) present[2] = true;
  for (int d = 0; d < 3; d++) {
    if (present[d]) {
      if (g.n[d] < 1) throw Error("grid needs at least one cell per direction");
      N[d] = g.n[d];
      ext[d] = N[d] + 1;
    }
    else {
      N[d] = 0;
      ext[d] = 1;
    }
  }
  // storage: last present direction fastest, each row padded to a multiple of
  // 32 points so rows start on 128-byte boundaries (FP32)
  fastdir = g.dim == 2 ? 1 : 2;
  int64_t pitch = (ext[fastdir] + 31) / 32 * 32;
  if (g.dim == 3) {
    stride[2] = 1;
    stride[1] = pitch;
    stride[0] = pitch * ext[1];
    nstore = stride[0] * ext[0];
  }
  else if (g.dim == 2) {
    stride[1] = 1;
    stride[0] = pitch;
    stride[2] = 0;
    nstore = pitch * ext[0];
  }
  else {
    stride[2] = 1;
    nstore = pitch;
  }
  ndense = (int64_t)ext[0] * ext[1] * ext[2];
  inva = 1.0 / g.a;
  dt = g.courant / g.a;

  // PML slabs: each PML region becomes its own chunk int(dx*a + 1 + 0.5) cells
  // thick (src/structure.cpp:509-523); coefficients per half-pixel position
  // (structure_chunk::use_pml, src/structure.cpp:627-691).
  for (int d = 0; d < 3; d++) {
    if (!present[d] || N[d] <= 1) continue;
    for (int s = 0; s < 2; s++) {
      double dx = g.pml_thickness[d][s];
      if (dx > 0) T[d][s] = int(dx * g.a + 1 + 0.5);
    }
    if (T[d][0] + T[d][1] >= N[d] && (T[d][0] > 0 || T[d][1] > 0))
      throw Error("PML slabs leave no interior chunk; make the cell larger");
    pml_dir[d] = T[d][0] > 0 || T[d][1] > 0;
  }
  for (int d = 0; d < 3; d++) {
    int np = 2 * N[d] + 2;
    sig[d].assign(np, 0.0);
    kap[d].assign(np, 1.0);
    siginv[d].assign(np, 1.0);
    if (!pml_dir[d]) continue;
    const double half_inva = 0.5 * inva;
    double bloc[2] = {g.io[d] * half_inva, (g.io[d] + 2 * N[d]) * half_inva};
    for (int pos = 0; pos < np; pos++) {
      int r = region(d, pos);
      if (r == 1) continue;
      int s = r == 0 ? 0 : 1;
      double dx = g.pml_thickness[d][s];
      double R = g.pml_R[d][s] > 0 ? g.pml_R[d][s] : 1e-15;
      double stretch = g.pml_stretch[d][s] > 0 ? g.pml_stretch[d][s] : 1.0;
      const double prefac = (-std::log(R)) / (4 * dx * (1. / 3.));
      const double kappa_prefac = (stretch - 1) / (1. / 4.);
      double x = pml_x(g.io[d] + pos, dx, bloc[s], g.a);
      if (x > 0) {
        double u = x / dx;
        double prof = u * u; // pml_quadratic_profile (src/structure.cpp:252-255)
        sig[d][pos] = 0.5 * dt * prefac * prof;
        kap[d][pos] = 1 + kappa_prefac * prof * (x / dx);
        siginv[d][pos] = 1 / (kap[d][pos] + sig[d][pos]);
      }
    }
  }

  // components, Yee shifts (src/meep/vec.hpp:1132-1140), updated ranges
  for (int c = 0; c < NC; c++) {
    have[c] = (g.components >> c) & 1;
    int t = ctype(c), dc = cdir(c);
    bool electric_like = (t == MFD_E || t == MFD_D);
    for (int d = 0; d < 3; d++) {
      int sh = 0;
      if (present[d]) sh = electric_like ? (d == dc) : (d != dc);
      shift[c][d] = sh;
      if (!present[d]) {
        klo[c][d] = khi[c][d] = 0;
      }
      else {
        // owned points 0 < s + 2k <= 2N; the high-wall points (s=0, k=N) are
        // zeroed by the metallic boundary after every update (zero_metal,
        // src/boundaries.cpp:190-203, 310-313), so they are never advanced.
        klo[c][d] = sh ? 0 : 1;
        khi[c][d] = N[d] - 1;
      }
    }
  }
  // D and B need their E/H partners allocated, and vice versa
  for (int c = 0; c < NC; c++)
    if (have[c]) {
      int t = ctype(c), d = cdir(c);
      int partner = t == MFD_E ? MFD_D : t == MFD_D ? MFD_E : t == MFD_H ? MFD_B : MFD_H;
      if (!have[comp(partner, d)]) throw Error("components must come in E/D and H/B pairs");
    }

  // curl plan (fields_chunk::figure_out_step_plan, src/fields.cpp:428-456;
  // step_db strides, src/step_db.cpp:44-130)
  for (int c = 0; c < NC; c++) {
    int t = ctype(c);
    if (!have[c] || (t != MFD_D && t != MFD_B)) continue;
    int d = cdir(c);
    int src_t = t == MFD_D ? MFD_H : MFD_E;
    int pd = cycle(d, 2), pderiv = cycle(d, 1); // plus component and its derivative
    int md = cycle(d, 1), mderiv = cycle(d, 2); // minus component and its derivative
    Curl &cp = curl[c];
    int g1 = (present[pderiv] && have[comp(src_t, pd)]) ? comp(src_t, pd) : -1;
    int g2 = (present[mderiv] && have[comp(src_t, md)]) ? comp(src_t, md) : -1;
    int64_t s1 = g1 >= 0 ? stride[pderiv] : 0, s2 = g2 >= 0 ? stride[mderiv] : 0;
    if (t == MFD_D) {
      s1 = -s1;
      s2 = -s2;
    }
    bool flip = false;
    int d1 = g1 >= 0 ? pderiv : -1, d2 = g2 >= 0 ? mderiv : -1;
    if (g1 < 0) {
      std::swap(g1, g2);
      std::swap(s1, s2);
      std::swap(d1, d2);
      flip = true;
    }
    cp.d1 = d1;
    cp.d2 = d2;
    cp.g1 = g1;
    cp.g2 = g2;
    cp.s1 = s1;
    cp.s2 = s2;
    cp.flip = flip;
    int ds0 = cycle(d, 1), du0 = cycle(d, 2);
    cp.dsig = pml_dir[ds0] ? ds0 : -1;
    cp.dsigu = pml_dir[du0] ? du0 : -1;
  }
}

int64_t Plan::store_index_of_dense(int64_t di) const {
  int k[3];
  dense_coords(di, k);
  return k[0] * stride[0] + k[1] * stride[1] + k[2] * stride[2];
}

Plan::ProbePoints Plan::center_probe(int d) const {
  ProbePoints pp;
  pp.n = 1;
  pp.idx[0] = 0;
  pp.w[0] = 1.0;
  const int c = comp(MFD_E, d);
  for (int e = 0; e < 3; e++) {
    if (!present[e]) continue;
    const int pc = N[e] - N[e] % 2; // icenter, relative to the low corner
    const int s = shift[c][e];
    int k0, nk;
    if ((pc - s) % 2 == 0) {
      k0 = (pc - s) / 2;
      nk = 1;
    }
    else {
      k0 = (pc - s - 1) / 2;
      nk = 2;
    }
    ProbePoints q;
    for (int i = 0; i < pp.n; i++)
      for (int j = 0; j < nk; j++) {
        const int k = k0 + j, pos = s + 2 * k;
        // a point no chunk owns reads as zero (fields::get_field(c, ivec))
        if (pos <= 0 || pos > 2 * N[e]) continue;
        q.idx[q.n] = pp.idx[i] + k * stride[e];
        q.w[q.n] = pp.w[i] * (nk == 2 ? 0.5 : 1.0);
        q.n++;
      }
    pp = q;
  }
  return pp;
}

void Plan::dense_coords(int64_t di, int k[3]) const {
  k[2] = int(di % ext[2]);
  di /= ext[2];
  k[1] = int(di % ext[1]);
  di /= ext[1];
  k[0] = int(di);
}

// Which chunks carry a conductivity array (structure_chunk::set_conductivity
// drops all-zero arrays per chunk, src/structure.cpp:868-905).  The chunk's
// array spans its cells' corner points k = c0..c1 along each direction.
void Plan::compute_cond_chunks(int c) {
  cond_chunk[c].assign(27, 0);
  if (cond[c].empty()) return;
  int lo[3][3], hi[3][3]; // [direction][region]
  for (int d = 0; d < 3; d++) {
    if (!present[d]) {
      for (int r = 0; r < 3; r++)
        lo[d][r] = hi[d][r] = 0;
      continue;
    }
    lo[d][0] = 0;
    hi[d][0] = T[d][0];
    lo[d][1] = T[d][0];
    hi[d][1] = N[d] - T[d][1];
    lo[d][2] = N[d] - T[d][1];
    hi[d][2] = N[d];
  }
  for (int rx = 0; rx < 3; rx++)
    for (int ry = 0; ry < 3; ry++)
      for (int rz = 0; rz < 3; rz++) {
        bool any = false;
        for (int kx = lo[0][rx]; kx <= hi[0][rx] && !any; kx++)
          for (int ky = lo[1][ry]; ky <= hi[1][ry] && !any; ky++)
            for (int kz = lo[2][rz]; kz <= hi[2][rz] && !any; kz++) {
              int64_t di = ((int64_t)kx * ext[1] + ky) * ext[2] + kz;
              if (cond[c][di] != 0.0) any = true;
            }
        cond_chunk[c][rx * 9 + ry * 3 + rz] = any;
      }
}

void Plan::plan_offdiag() {
  any_offdiag = false;
  for (int d = 0; d < 3; d++) {
    OffDiag &od = offdiag[d];
    od = OffDiag();
    const int ec = comp(MFD_E, d);
    if (!have[ec]) continue;
    int dir[2] = {cycle(d, 1), cycle(d, 2)};
    bool g[2], u[2];
    for (int q = 0; q < 2; q++) {
      g[q] = have[comp(MFD_D, dir[q])];
      u[q] = false;
      if (g[q])
        for (double v : chi1inv[ec][dir[q]])
          if (v != 0.0) {
            u[q] = true;
            break;
          }
    }
    if ((!g[0] && g[1]) || (g[0] && g[1] && !u[0] && u[1])) {
      std::swap(dir[0], dir[1]);
      std::swap(u[0], u[1]);
    }
    if (u[0]) od.dir[od.n++] = dir[0];
    if (u[0] && u[1]) od.dir[od.n++] = dir[1];
    any_offdiag = any_offdiag || od.n > 0;
  }
}

void Plan::set_bloch(const int per[3], const double k[3]) {
  complex_fields = false;
  for (int d = 0; d < 3; d++) {
    periodic[d] = present[d] && per[d] != 0;
    eikna[d] = std::complex<double>(1, 0);
    if (!periodic[d]) continue;
    // the Brillouin-zone edge exactly: eikna = -1 (src/boundaries.cpp:98-103)
    if (k[d] * N[d] == 0.5 * g.a) eikna[d] = std::complex<double>(-1.0, 0.0); // -exp(-Im k ...), k real
    else eikna[d] = std::exp(std::complex<double>(0.0, 1.0) * std::complex<double>(k[d], 0.0) * ((2 * pi / g.a) * N[d]));
    if (k[d] != 0.0) complex_fields = true;
    // shift-0 components own the high-wall points (no metal there)
    for (int c = 0; c < NC; c++)
      if (present[d] && shift[c][d] == 0) khi[c][d] = N[d];
  }
}

} // namespace mfd


namespace mfd {

/* ------------------------------------------------------- material grids */
void Plan::matgrid_box(int id, int c, int lo[3], int hi[3]) const {
  const MatGridSpec &s = matgrids[id].spec;
  for (int d = 0; d < 3; d++) {
    if (!present[d]) {
      lo[d] = hi[d] = 0;
      continue;
    }
    const double a2 = 2.0 * g.a;
    const double k0 = ((s.center[d] - 0.5 * s.size[d]) * a2 - g.io[d] - shift[c][d]) / 2;
    const double k1 = ((s.center[d] + 0.5 * s.size[d]) * a2 - g.io[d] - shift[c][d]) / 2;
    lo[d] = std::max(0, int(std::floor(k0)) - 1);
    hi[d] = std::min(N[d], int(std::ceil(k1)) + 1);
  }
}

int Plan::matgrid_at(int c, const int k[3]) const {
  double x[3];
  point_coords(c, k, x);
  for (int id = int(matgrids.size()) - 1; id >= 0; id--)
    if (mg_inside(matgrids[id].spec, x)) return id;
  return -1;
}

void Plan::apply_matgrids_host() {
  for (int id = 0; id < int(matgrids.size()); id++) {
    const MatGrid &mg = matgrids[id];
    for (int d = 0; d < 3; d++) {
      const int c = comp(MFD_E, d);
      if (!have[c]) continue;
      std::vector<double> &chi = chi1inv[c][d];
      if (chi.empty()) chi.assign(ndense, 1.0);
      int lo[3], hi[3], k[3];
      matgrid_box(id, c, lo, hi);
      for (k[0] = lo[0]; k[0] <= hi[0]; k[0]++)
        for (k[1] = lo[1]; k[1] <= hi[1]; k[1]++)
          for (k[2] = lo[2]; k[2] <= hi[2]; k[2]++) {
            double x[3], r[3];
            point_coords(c, k, x);
            if (!mg_inside(mg.spec, x)) continue;
            mg_coords(mg.spec, x, r);
            const double up = mg_project(mg_interp(mg.u.data(), mg.spec.n, r), mg.spec.beta, mg.spec.eta);
            chi[(int64_t(k[0]) * ext[1] + k[1]) * ext[2] + k[2]] = 1.0 / mg_eps(mg.spec, d, up);
          }
    }
  }
}

void Plan::matgrid_vjp_host(int id, const std::vector<int> &comps, const int lo[3], const int hi[3],
                            const double *gchi, double *gu) const {
  const MatGrid &mg = matgrids[id];
  const MatGridSpec &s = mg.spec;
  const int64_t nu = int64_t(s.n[0]) * s.n[1] * s.n[2];
  std::fill(gu, gu + nu, 0.0);
  int64_t q = 0;
  for (int c : comps) {
    const int d = c % 3;
    int k[3];
    for (k[0] = lo[0]; k[0] <= hi[0]; k[0]++)
      for (k[1] = lo[1]; k[1] <= hi[1]; k[1]++)
        for (k[2] = lo[2]; k[2] <= hi[2]; k[2]++, q++) {
          if (gchi[q] == 0.0 || matgrid_at(c, k) != id) continue;
          double x[3], r[3];
          point_coords(c, k, x);
          mg_coords(s, x, r);
          const double rho = mg_interp(mg.u.data(), s.n, r);
          const double eps = mg_eps(s, d, mg_project(rho, s.beta, s.eta));
          const double grho = gchi[q] * (-(s.eps2[d] - s.eps1[d]) / (eps * eps)) *
                              mg_project_deriv(rho, s.beta, s.eta);
          int i1[3], i2[3];
          double w[3];
          for (int e = 0; e < 3; e++)
            mg_map(r[e], s.n[e], i1[e], i2[e], w[e]);
          for (int a = 0; a < 2; a++)
            for (int b = 0; b < 2; b++)
              for (int cc = 0; cc < 2; cc++) {
                const int x0 = a ? i2[0] : i1[0], y0 = b ? i2[1] : i1[1], z0 = cc ? i2[2] : i1[2];
                const double wt = (a ? w[0] : 1.0 - w[0]) * (b ? w[1] : 1.0 - w[1]) * (cc ? w[2] : 1.0 - w[2]);
                gu[(int64_t(x0) * s.n[1] + y0) * s.n[2] + z0] += grho * wt;
              }
        }
  }
}

} // namespace mfd
