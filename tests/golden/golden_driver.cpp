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
