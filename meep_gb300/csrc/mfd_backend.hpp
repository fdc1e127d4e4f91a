// Interface between the C ABI (mfd_capi.cpp) and an execution backend.  The
// product links the CUDA backend (mfd_cuda_*.cu); the CPU oracle used by the
// tests implements the same interface in oracle/cpu_backend.cpp.
#pragma once

#include <complex>
#include <vector>

#include "mfd_plan.hpp"

namespace mfd {

// Source amplitudes of one source time function for one full step, taken at
// the times fields::step() calls calc_sources (src/step.cpp:64-108).
struct SrcStepValues {
  std::complex<double> cur_b; // current at t*dt            (step_source(B))
  std::complex<double> cur_d; // current at (t+1/2)*dt      (step_source(D))
  std::complex<double> dip_e; // dipole  at (t+1)*dt        (integrated E sources)
};

// Near-to-far transform: one equivalent current sheet per DFT monitor.  The
// monitor holds the DFT of one tangential field on its own Yee grid with the
// sheet's sign, surface weight and dV folded in (fields::add_dft_near2far,
// src/near2far.cpp:569-651); point k of the monitor box sits at
// (is_half + k) * inva + rshift (IVEC_LOOP_LOC plus the lattice-image shift).
struct N2FSheet {
  int id;            // DFT monitor
  int c0;            // equivalent current: 0..2 electric x, y, z; 3..5 magnetic
  double is_half[3]; // half the loop-start ivec of the monitor's first point
  double rshift[3];  // lattice-image shift of the points
};
struct N2FSpec {
  int dim;         // 2 (green2d) or 3 (green3d)
  double eps, mu;  // homogeneous medium around the sheets
  double inva;     // grid spacing 1/a
  int pdir[2];     // periodic image directions, -1 none
  int pn[2];       // images -pn..pn along each
  double pk[2];    // Bloch phase per image
  double period[2];
};

class Backend {
public:
  virtual ~Backend() {}
  // Allocate fields and upload materials, PML tables and sources.
  virtual void setup(Plan &p) = 0;
  // Upload monitor p.monitors[id] (may be called after setup).
  virtual void add_monitor(Plan &p, int id) = 0;
  // One full step from step count t to t+1, then the DFT updates at t+1.
  virtual void step(Plan &p, int64_t t, const std::vector<SrcStepValues> &vals) = 0;
  virtual void get_field(Plan &p, int c, double *out_dense) = 0;
  // imaginary part of a complex (Bloch) field
  virtual void get_field_im(Plan &p, int c, double *out_dense) = 0;
  virtual void get_dft(Plan &p, int id, double *out) = 0;
  virtual void flux(Plan &p, int npairs, const int *idE, const int *idH, double *out) = 0;
  // replace the DFT sums of monitor id (npts * nfreq complex, re/im)
  virtual void set_dft(Plan &p, int id, const double *in) = 0;
  // multiply the DFT sums of monitor id by s (dft_chunk::scale_dft)
  virtual void scale_dft(Plan &p, int id, std::complex<double> s) = 0;
  // far fields (6 complex values per far point and frequency, point-major,
  // then frequency, then Ex..Hz, re/im interleaved) of the sheets at the nx
  // points x (3 coordinates each)
  virtual void farfield(Plan &p, const N2FSpec &s, const std::vector<N2FSheet> &sheets, int64_t nx, const double *x,
                        double *out) = 0;
  virtual void synchronize() {}
  virtual long long launches() const { return 0; }
  virtual double last_step_ms() const { return 0.0; }
  // called before a batch of steps / after it (for timing)
  virtual void begin_steps() {}
  virtual void end_steps() {}

  // ---- differentiation: reverse-time (discrete) adjoint of the step ----
  // Design = E components `comps` over the point box lo..hi of each.
  virtual void set_design(Plan &p, const std::vector<int> &comps, const int lo[3], const int hi[3]) {
    (void)p, (void)comps, (void)lo, (void)hi;
    throw Error("this backend has no adjoint");
  }
  // buffer for the design-box D of `nslots` steps; record after a step
  virtual void alloc_record(Plan &p, int64_t nslots) { (void)p, (void)nslots; }
  virtual void record_design(Plan &p, int64_t slot) { (void)p, (void)slot; }
  // full-state checkpoints (all fields and auxiliaries, no DFT sums)
  virtual int snapshot(Plan &p) {
    (void)p;
    return -1;
  }
  virtual void restore(Plan &p, int slot) { (void)p, (void)slot; }
  virtual void set_skip_dft(bool skip) { (void)skip; }
  // adjoint sweep: begin (zero adjoint fields, upload dJ/dDFT of the listed
  // monitors), one reversed step s (state s -> s+1, recorded D of step s at
  // `slot`), end (gradient dJ/dchi1inv per design component and box point)
  virtual void adjoint_begin(Plan &p, int nmon, const int *ids, const double *const *grads) {
    (void)p, (void)nmon, (void)ids, (void)grads;
  }
  virtual void adjoint_step(Plan &p, int64_t s, int64_t slot) { (void)p, (void)s, (void)slot; }
  virtual void adjoint_end(Plan &p, double *grad) { (void)p, (void)grad; }
  // dJ/du of material grid `id` from dJ/dchi1inv over the design box
  // (mfd_material_grid_vjp); the oracle evaluates it on the host
  virtual void matgrid_vjp(Plan &p, int id, const std::vector<int> &comps, const int lo[3], const int hi[3],
                           const double *gchi, double *gu) {
    p.matgrid_vjp_host(id, comps, lo, hi, gchi, gu);
  }
};

// Defined by whichever backend is linked in.
Backend *make_backend(const Plan &p);
// mfd_subpixel_rows (arguments checked by the C ABI)
void subpixel_rows(int dim, int cdir, int64_t npix, const double *lo, const double *hi, double tol, int maxeval,
                   int nobj, const mfd_object *objs, double eps_default, double *rows);
// mfd_green (arguments checked by the C ABI)
void green_eval(int dim, int c0, double freq, double eps, double mu, double f0re, double f0im, int64_t n,
                const double *x, const double *x0, double *out);

} // namespace mfd
