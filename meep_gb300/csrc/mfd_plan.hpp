// Host-side description of one FDTD problem on a single global Yee grid.
//
// The reference splits the cell into chunks: one per PML slab and one for the
// interior (src/structure.cpp:96-149, effort volumes :509-523), exchanges the
// not-owned points between chunks every half step (src/step.cpp:225-287) and
// picks the update formula per chunk (PML or not, src/step_db.cpp:54-60,
// src/update_eh.cpp:159-160).  Here the whole cell is one device-resident
// array per component; the chunk a point would belong to is recomputed from its
// half-pixel coordinate (Plan::region), so every point is advanced with the
// same formula and coefficients as in the reference, and no halo copies are
// needed at all.
#pragma once

#include <complex>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "mfd.h"
#include "matgrid.hpp"

namespace mfd {

constexpr int NC = MFD_NCOMP;
constexpr int MAX_POLES = 4;

inline int ctype(int c) { return c / 3; }
inline int cdir(int c) { return c % 3; }
inline int comp(int t, int d) { return 3 * t + d; }
// cycle_direction for Cartesian directions (src/meep/vec.hpp:586-589)
inline int cycle(int d, int s) { return (d + s) % 3; }

struct Error : std::runtime_error {
  explicit Error(const std::string &m) : std::runtime_error("meep: " + m) {}
};

// Source time dependence: Gaussian (both reference constructors) or CW with a
// tanh turn-on.  dipole()/current() follow src/sources.cpp:72-110 and
// src/meep.hpp:978-991 (current is the finite difference of the dipole).
struct SrcTime {
  int kind = 0; // 0 gaussian, 1 continuous
  double freq = 0, fwidth = 0, width = 0, peak_time = 0, cutoff = 0;
  std::complex<double> cfreq{0, 0};
  double start = 0, end = 0, slowness = 3;
  bool integrated = true;
  // cached values of the last update (src_time::update)
  double cur_time = -1e300;
  std::complex<double> cur_dipole{0, 0}, cur_current{0, 0};

  static SrcTime gaussian(double f, double fw, double s = 5.0);
  static SrcTime gaussian_window(double f, double w, double st, double et);
  static SrcTime continuous(std::complex<double> f, double w, double st, double et, double s);
  std::complex<double> dipole(double t) const;
  std::complex<double> current(double t, double dt) const {
    return (dipole(t + dt) - dipole(t)) / dt;
  }
  void update(double t, double dt) {
    if (t != cur_time) {
      cur_dipole = dipole(t);
      cur_current = current(t, dt);
      cur_time = t;
    }
  }
  // bandwidth used by the automatic DFT decimation (src/dft.cpp:196-217)
  double get_fwidth() const { return kind == 0 ? fwidth : 0.0; }
  double frequency_re() const { return kind == 0 ? freq : cfreq.real(); }
};

// One source point list on component c (E or H); ft2 = D or B receives it.
struct SourceGroup {
  int c = 0;
  int src = 0;
  std::vector<int64_t> idx; // dense indices
  std::vector<std::complex<double>> amp;
};

struct Pole {
  int ft = MFD_E;
  double omega0 = 0, gamma = 0;
  bool drude = false;
  std::vector<double> sigma[3]; // dense per E component direction; empty = absent
};

struct Monitor {
  int c = 0;
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  std::vector<double> w[3]; // per present direction
  double dV = 1.0;
  bool include_weights = true;
  bool sqrt_weights = false; // the square root of the weight product (sqrt_dV_and_interp_weights)
  std::complex<double> scale{1, 0};
  bool centered = false;
  std::vector<double> freq;
  int decimation = 1;
  size_t npts = 0;
};

class Plan {
public:
  mfd_grid g{};
  bool present[3] = {false, false, false};
  int N[3] = {0, 0, 0};
  int ext[3] = {1, 1, 1};
  int64_t stride[3] = {0, 0, 0};
  int64_t ndense = 1, nstore = 1;
  int fastdir = 2;
  double dt = 0, inva = 0;
  int T[3][2] = {{0, 0}, {0, 0}, {0, 0}}; // PML slab thickness in cells
  bool pml_dir[3] = {false, false, false};
  std::vector<double> sig[3], kap[3], siginv[3]; // indexed by half-pixel pos 0..2N+1
  bool have[NC] = {};
  int shift[NC][3] = {};
  int klo[NC][3] = {}, khi[NC][3] = {}; // updated (owned, not on a metal wall) range

  // Bloch-periodic directions (fields::use_bloch, src/boundaries.cpp:90-109):
  // the not-owned points (position 0 of shift-0 components, 2N+1 of shift-1
  // components) hold the field of the opposite side times conj(eikna) /
  // eikna, eikna = exp(2 pi i k L); the shift-0 high-wall points are owned
  bool periodic[3] = {false, false, false};
  std::complex<double> eikna[3] = {{1, 0}, {1, 0}, {1, 0}};
  bool complex_fields = false; // a periodic direction with k != 0
  void set_bloch(const int per[3], const double k[3]);
  bool any_periodic() const { return periodic[0] || periodic[1] || periodic[2]; }

  // curl plan (D, B components): f -= dtdx (g1[i+s1]-g1[i] + g2[i]-g2[i+s2])
  struct Curl {
    int g1 = -1, g2 = -1;
    int64_t s1 = 0, s2 = 0;
    bool flip = false; // dtdx negated (g1 missing, g2 moved into its place)
    int d1 = -1, d2 = -1; // directions of the strides s1, s2
    int dsig = -1, dsigu = -1;
  } curl[NC];

  // material data (dense arrays, double)
  std::vector<double> chi1inv[NC][3];
  std::vector<double> cond[NC];                     // D/B components
  std::vector<uint8_t> cond_chunk[NC];              // 27 flags: chunk has nonzero cond
  std::vector<Pole> poles;                          // reference list order (last added first)
  std::vector<SrcTime> srcs;
  std::vector<SourceGroup> sources;
  std::vector<Monitor> monitors;

  // Off-diagonal inverse-permittivity terms of the E update: for E along d,
  // E = chi_dd (D-P)_d + OFFDIAG over the D components along dir[0], dir[1]
  // (in this order), each the 4-point average of that D component around
  // the E point weighted by chi_d,dir at the two E-direction neighbours
  // (src/update_eh.cpp:179-192; swap rule and OFFDIAG
  // src/step_generic.cpp:574-582).  An entry counts when its array holds a
  // nonzero value.  Set by plan_offdiag() once the materials are final.
  struct OffDiag {
    int n = 0;
    int dir[2] = {-1, -1};
  } offdiag[3];
  bool any_offdiag = false;
  void plan_offdiag();

  explicit Plan(const mfd_grid &grid);

  // chunk region of half-pixel position pos along d: 0 low slab, 1 interior, 2 high slab
  int region(int d, int pos) const {
    if (!present[d]) return 1;
    if (T[d][0] > 0 && pos <= 2 * T[d][0]) return 0;
    if (T[d][1] > 0 && pos > 2 * (N[d] - T[d][1])) return 2;
    return 1;
  }
  bool in_slab(int d, int pos) const { return region(d, pos) != 1; }

  // Divergence test of fields::step(): the reference aborts with "simulation
  // fields are NaN or Inf" when get_field(D_EnergyDensity, gv.center()) is
  // not finite (src/step.cpp:137-138), i.e. half the sum over the E
  // components of E_d * D_d, each interpolated at the cell centre
  // (src/monitor.cpp:76-91).  The centre is io + n rounded down to even
  // (grid_volume::icenter, src/vec.cpp:1089-1101); a component reads the one
  // or two Yee points around it per direction with weights 1 or 1/2, and
  // drops zero weights (grid_volume::interpolate, src/vec.cpp:558-598).
  // Returns the store indices and weights for E component direction d
  // (the D component at the same Yee positions uses the same ones).
  struct ProbePoints {
    int n = 0;
    int64_t idx[8] = {};
    double w[8] = {};
  };
  ProbePoints center_probe(int d) const;

  // Material grids (mfd_add_material_grid): at setup every E-component Yee
  // point inside a grid's block takes the diagonal chi1inv 1 / eps of the
  // projected, interpolated weights (matgrid.hpp), grids applied in the
  // order added (a later one wins where blocks overlap, as the last object
  // of a geometry does).  The CUDA engine evaluates them on the device; the
  // CPU oracle through apply_matgrids_host.
  struct MatGrid {
    MatGridSpec spec;
    std::vector<double> u; // n0 * n1 * n2, row-major
  };
  std::vector<MatGrid> matgrids;
  // physical coordinates of point k of component c: (io + shift + 2k) / (2a)
  void point_coords(int c, const int k[3], double x[3]) const {
    for (int d = 0; d < 3; d++)
      x[d] = present[d] ? double(g.io[d] + shift[c][d] + 2 * k[d]) * (0.5 * inva) : 0.0;
  }
  // index box of component c that holds every point of grid id's block
  // (the kernels test each point exactly)
  void matgrid_box(int id, int c, int lo[3], int hi[3]) const;
  // the grid id that sets point k of E component c (-1: none)
  int matgrid_at(int c, const int k[3]) const;
  void apply_matgrids_host();
  // dJ/du of grid id from dJ/dchi1inv over a design box (mfd_backward's
  // layout: per design component, the box points x-major)
  void matgrid_vjp_host(int id, const std::vector<int> &comps, const int lo[3], const int hi[3],
                        const double *gchi, double *gu) const;
  int64_t dense_count() const { return ndense; }
  int64_t store_index_of_dense(int64_t di) const;
  void dense_coords(int64_t di, int k[3]) const;
  void compute_cond_chunks(int c);
};

} // namespace mfd
