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
};

// Defined by whichever backend is linked in.
Backend *make_backend(const Plan &p);
// mfd_subpixel_rows (arguments checked by the C ABI)
void subpixel_rows(int dim, int cdir, int64_t npix, const double *lo, const double *hi, double tol, int maxeval,
                   int nobj, const mfd_object *objs, double eps_default, double *rows);

} // namespace mfd
