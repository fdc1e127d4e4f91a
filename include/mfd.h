/* mfd.h -- C ABI of the GB300 FDTD stepping engine (drop-in for Meep's
 * fields::step() path).
 *
 * All entry points return 0 on success and a negative status on failure;
 * mfd_last_error() then holds a message ("meep: ..." style, like the
 * reference's meep::abort, src/mympi.cpp:238-254).  Handles are opaque and
 * not thread-safe (the reference API is not thread-safe either,
 * src/meep.hpp:1621-1622); each handle owns one CUDA stream.
 *
 * Conventions
 *   component  c = 3*type + direction, type E=0 H=1 D=2 B=3, direction X=0 Y=1 Z=2
 *              (the reference's enum component orders Ex..Bz with cylindrical
 *              slots in between, src/meep/vec.hpp:31-56; the C++ drop-in maps it)
 *   grid       dim 1 uses Z only, dim 2 uses X and Y, dim 3 uses X, Y, Z
 *              (reference: src/meep/vec.hpp ndim / LOOP_OVER_DIRECTIONS).
 *              Every component array has n[d]+1 points along each present
 *              direction; point k of component c sits at half-pixel coordinate
 *              io[d] + shift_c[d] + 2k (shift = Yee offset, src/meep/vec.hpp:1132-1140).
 *   arrays     exchanged through this ABI are dense, x slowest, the last present
 *              direction fastest, (n[d]+1) per present direction, float64.
 *   precision  64: fields and coefficients in double; 32: float storage and
 *              arithmetic for fields/coefficients, DFT sums kept in double.
 */
#ifndef MFD_ABI_H_
#define MFD_ABI_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mfd_sim mfd_sim;

enum { MFD_E = 0, MFD_H = 1, MFD_D = 2, MFD_B = 3 };
enum { MFD_X = 0, MFD_Y = 1, MFD_Z = 2 };
enum { MFD_NCOMP = 12 };

/* Grid and boundary description.
 * Replaces: structure(grid_volume, material_function&, boundary_region, ...)
 *           src/meep.hpp:830-839, with pml() src/meep.hpp:732-737 and the
 *           quadratic profile of src/structure.cpp:252-255. */
typedef struct mfd_grid {
  int dim;                    /* 1, 2 or 3 */
  int n[3];                   /* cells per direction (X, Y, Z); 0 for absent */
  int io[3];                  /* half-pixel coordinate of the low corner */
  double a;                   /* resolution (pixels per unit length) */
  double courant;             /* dt = courant / a */
  double pml_thickness[3][2]; /* [direction][0=low,1=high]; 0 = no PML */
  double pml_R[3][2];         /* asymptotic reflection (reference default 1e-15) */
  double pml_stretch[3][2];   /* mean stretch (reference default 1.0) */
  int precision;              /* 64 or 32 */
  int components;             /* bit mask of allocated components (bit c) */
} mfd_grid;

/* Create / destroy.  Replaces fields::fields(structure*, ...) src/meep.hpp:1740-1742.
 * Fields start at zero at t = 0, real fields (fields::use_real_fields). */
int mfd_create(const mfd_grid *grid, mfd_sim **out);
void mfd_destroy(mfd_sim *sim);
const char *mfd_last_error(void);

/* Inverse permittivity row entry chi1inv[c][d] for E component c (dense
 * component-grid array).  Replaces structure_chunk::set_chi1inv
 * src/anisotropic_averaging.cpp:211.  Off-diagonal entries (d != dir(c)) use
 * the reference's 4-point averaging (src/step_generic.cpp:580-581). */
int mfd_set_chi1inv(mfd_sim *sim, int c, int d, const double *values);

/* Conductivity of D or B component c (dense array); condinv = 1/(1+sigma dt/2).
 * Replaces structure_chunk::set_conductivity src/structure.cpp:868-905 and
 * update_condinv src/structure.cpp:693-707. */
int mfd_set_conductivity(mfd_sim *sim, int c, const double *values);

/* Lorentzian / Drude pole on E (field_type E).  sigma[d] is the dense sigma
 * array of E component d (NULL if the component is absent).  Poles are applied
 * in the reference's list order (last added first).  Replaces
 * structure::add_susceptibility src/structure.cpp:477-507 with
 * lorentzian_susceptibility src/susceptibility.cpp:188-281. */
int mfd_add_lorentzian(mfd_sim *sim, int field_type, double omega0, double gamma, int drude,
                       const double *const sigma[3]);

/* Source time functions.  Replaces gaussian_src_time src/sources.cpp:72-110
 * (both constructors) and continuous_src_time.  With explicit_window == 0 the
 * Gaussian is gaussian_src_time(freq, fwidth, s) with s = start (0 means the
 * default 5); otherwise gaussian_src_time(freq, width, start, end).
 * Returns id >= 0 in *id. */
int mfd_add_gaussian_src(mfd_sim *sim, double freq, double fwidth_or_width, double start,
                         double end, int explicit_window, int is_integrated, int *id);
int mfd_add_continuous_src(mfd_sim *sim, double freq_re, double freq_im, double width,
                           double start, double end, double slowness, int is_integrated,
                           int *id);

/* Current of source time function src_id at `time` as fields::step takes it
 * from src_time::update (the difference quotient (dipole(time + dt) -
 * dipole(time)) / dt, src/sources.cpp); out = (re, im).  Host arithmetic, for
 * callers that integrate the source spectrum (dft_ldos::update,
 * src/dft_ldos.cpp:157-162). */
int mfd_src_current(const mfd_sim *sim, int src_id, double time, double *out);

/* Point list of a source on component c (an E or H component: the current is
 * applied to the D or B field of that direction).  idx are dense-array linear
 * indices, amp interleaved (re, im).  Replaces fields::add_volume_source /
 * src_vol src/sources.cpp:223-312, src/meep_internals.hpp:49-82. */
int mfd_add_source_points(mfd_sim *sim, int c, int src_id, size_t npts, const int64_t *idx,
                          const double *amp);

/* DFT monitor on component c over the box lo[d]..hi[d] (point indices of the
 * component grid, inclusive).  w[d] holds hi[d]-lo[d]+1 per-point weights for
 * each present direction (the reference's IVEC_LOOP_WEIGHT factors), dV the
 * volume element, scale the complex stored weight.  include_weights: 0 none,
 * 1 the weight product, 2 its square root (sqrt_dV_and_interp_weights, used
 * by the diagonal stress-tensor terms of add_dft_force).  centered != 0 averages the
 * Yee values onto the centred grid (yee2cent_offsets).  Replaces
 * fields::add_dft src/dft.cpp:175-235 / dft_chunk src/dft.cpp:266-308.
 * Returns monitor id in *id. */
int mfd_add_dft(mfd_sim *sim, int c, const int lo[3], const int hi[3], const double *const w[3],
                double dV, int include_weights, double scale_re, double scale_im, int centered,
                size_t nfreq, const double *freq, int decimation, int *id);

/* Advance n full time steps (fields::step, src/step.cpp:35-139).  Returns
 * once the steps are queued on the GPU (a call whose steps ran a divergence
 * probe waits for it); the calls that read results wait for them. */
int mfd_step(mfd_sim *sim, int n);

/* Current step count t (fields::t) and dt. */
int mfd_get_time(const mfd_sim *sim, int64_t *t, double *dt);

/* Copy the dense array of component c to host doubles. */
int mfd_get_field(mfd_sim *sim, int c, double *out);

/* Copy monitor `id` sums to host: npts*nfreq*(re,im), point-major. */
int mfd_get_dft(mfd_sim *sim, int id, double *out, size_t *npts, size_t *nfreq);

/* Flux spectrum sum_k Re(E_k conj(H_k)) over paired monitors (E[i], H[i]),
 * accumulated in double on the device.  Replaces dft_flux::flux
 * src/dft.cpp:542-556. out has nfreq entries. */
int mfd_flux(mfd_sim *sim, int npairs, const int *idE, const int *idH, double *out);

/* Replace the sums of monitor `id` by in (npts*nfreq*(re,im), the layout of
 * mfd_get_dft).  Replaces the chunk loop of _load_dft_data
 * python/meep.i:511-527 (Simulation.load_flux_data / load_minus_flux_data);
 * sums accumulated by later steps add to these values. */
int mfd_set_dft(mfd_sim *sim, int id, const double *in);

/* Multiply the sums of monitor `id` by (s_re + i s_im).  Replaces
 * dft_chunk::scale_dft src/dft.cpp:402-406 (dft_near2far::scale_dfts
 * src/near2far.cpp:124-126, dft_flux::scale_dfts). */
int mfd_scale_dft(mfd_sim *sim, int id, double s_re, double s_im);

/* ---- Near-to-far transform ----
 * Far fields of equivalent current sheets.  Each of the nsheet monitors
 * ids[i] holds the DFT of one tangential field on its own Yee grid (centered
 * = 0) with the sheet's sign and surface weight in its scale and include
 * weights on (how fields::add_dft_near2far src/near2far.cpp:569-651 adds
 * them); src_comp[i] is the equivalent current it stands for (mfd component
 * code of Ex..Ez or Hx..Hz); point k of the monitor box sits at
 * (is_half[3i+d] + k_d) / a + rshift[3i+d] (the loop-start ivec / 2 of its
 * first point and the lattice-image shift).  eps, mu: the homogeneous medium.
 * periodic_dir[j] (0..2, or -1) with periodic_n[j] images on each side,
 * periodic_k[j] phase per image and period[j] (the Nperiods sum of
 * add_dft_near2far).  x: nx far points (x, y, z; z ignored in 2-D).  out:
 * nx * nfreq * 6 complex values (re, im), far point slowest, then frequency,
 * then Ex, Ey, Ez, Hx, Hy, Hz.  All monitors must have the same frequencies.
 * 2-D (x, y) and 3-D grids.  Replaces dft_near2far::farfield_lowlevel
 * src/near2far.cpp:334-378 for a list of far points. */
int mfd_farfield(mfd_sim *sim, int nsheet, const int *ids, const int *src_comp, const double *is_half,
                 const double *rshift, double eps, double mu, const int periodic_dir[2], const int periodic_n[2],
                 const double periodic_k[2], const double period[2], int64_t nx, const double *x, double *out);

/* The homogeneous-medium Green's function for n point pairs: out[12 i ..]
 * = the 6 complex fields (Ex..Hz, re/im) at x[3i..] of a current f0 of
 * component c0 (mfd code of Ex..Ez, Hx..Hz) at x0[3i..].  dim 3: green3d
 * src/near2far.cpp:131-181; dim 2: green2d src/near2far.cpp:201-245 (x, y
 * only; c0 of any direction).  No mfd_sim needed. */
int mfd_green(int dim, int c0, double freq, double eps, double mu, double f0_re, double f0_im, int64_t n,
              const double *x, const double *x0, double *out);

/* ---- Differentiation: reverse-time adjoint of the leapfrog update ----
 * Design = the inverse-permittivity diagonal chi1inv of E components `comps`
 * over the point box lo..hi (inclusive, component-grid indices).
 * mfd_forward advances n steps like mfd_step and keeps what the adjoint needs:
 * with checkpoint_every == 0 it records D at the design points for every step;
 * with checkpoint_every = K > 0 it stores a full-state checkpoint every K steps
 * and the backward pass recomputes each segment from its checkpoint (sqrt(T)
 * memory); checkpoint_every = -1 picks recording when it fits a memory budget
 * (16 GB, or MFD_RECORD_BUDGET_GB) and sqrt(nsteps) checkpoints otherwise.  mfd_backward takes dJ/dDFT for the listed monitors (per monitor
 * npts*nfreq*(re,im) = dJ/dRe F + i dJ/dIm F) and returns dJ/dchi1inv for every
 * design component and box point (ncomp * npts doubles, x slowest).
 * Replaces the frequency-domain gradient of the reference's adjoint solver
 * (python/adjoint/optimization_problem.py:262-393, src/meepgeom.cpp:2835-3011)
 * with the exact gradient of the time-stepped problem.  After mfd_backward the
 * fields hold an intermediate state; create a new handle for another run.
 * Not supported with dispersive materials or conductivity. */
int mfd_design(mfd_sim *sim, int ncomp, const int *comps, const int lo[3], const int hi[3]);
int mfd_forward(mfd_sim *sim, int nsteps, int checkpoint_every);
int mfd_backward(mfd_sim *sim, int nmon, const int *mon_ids, const double *const *dft_grad,
                 double *grad_chi1inv);

/* Material grid (replaces the MaterialGrid material of a Block: the weights
 * interpolated by material_grid_val / matgrid_val, src/meepgeom.cpp:489-540,
 * projected by tanh_projection, :497-502, and mapped to eps by
 * epsilon_material_grid, :569-581; python/geom.py MaterialGrid).  Every
 * E-component Yee point x inside the axis-aligned block |x - center| <=
 * size / 2 (per direction) takes the diagonal chi1inv
 *   1 / (eps1[d] + p (eps2[d] - eps1[d])),  p = tanh_projection(u(r), beta, eta),
 * u(r) the linear interpolation of the weights (n[0] x n[1] x n[2], row-major,
 * nodes at cell centres, mirror faces: linear_interpolate, src/fields.cpp:
 * 792-806) at r = 0.5 + (x - center) / size (0 along a zero-size direction).
 * Grids apply in the order added, over the chi1inv arrays, at the first step;
 * the CUDA engine evaluates them on the device.  Default grid type only (no
 * overlap rule), no subpixel smoothing of the grid (do_averaging false, the
 * reference's default), weights in [0, 1], beta >= 0 (may be infinite), eta
 * in [0, 1].  *id receives the grid's index.
 *
 * mfd_material_grid_vjp: dJ/du of grid `id` (n[0]*n[1]*n[2] doubles) from
 * dJ/dchi1inv of the E components `comps` over the point box lo..hi
 * (mfd_backward's layout: per component, the box points x slowest), through
 * the projection and the interpolation (the chain material_grids_addgradient
 * forms by finite differences, src/meepgeom.cpp:2626-2756); points another,
 * later grid covers do not count. */
int mfd_add_material_grid(mfd_sim *sim, const double center[3], const double size[3], const int n[3],
                          const double *weights, double beta, double eta, const double eps1[3],
                          const double eps2[3], int *id);
int mfd_material_grid_vjp(mfd_sim *sim, int id, int ncomp, const int *comps, const int lo[3], const int hi[3],
                          const double *grad_chi1inv, double *grad_weights);

/* Bloch-periodic boundaries (replaces fields::use_bloch, src/boundaries.cpp:
 * 90-109): directions with periodic[d] != 0 get the Bloch wavevector k[d]
 * (units of 2 pi / a); the other directions keep metallic walls.  A nonzero
 * k makes the fields complex (fields::use_real_fields then aborts in the
 * reference); mfd_get_field returns the real part, mfd_get_field_im the
 * imaginary part.  Before the first step; PML may sit in front of a
 * periodic wall. */
int mfd_set_bloch(mfd_sim *s, const int periodic[3], const double k[3]);
int mfd_get_field_im(mfd_sim *s, int c, double *out);

/* Subpixel averaging of a geometry on the GPU.  The reference computes the
 * averaged inverse-permittivity rows on the host, pixel by pixel
 * (structure_chunk::set_chi1inv -> material_function::eff_chi1inv_row,
 * src/anisotropic_averaging.cpp:87-324); this evaluates the same rows for
 * npix pixels at once, one GPU thread per pixel, for a geometry of blocks,
 * spheres and cylinders with scalar permittivities (the last object
 * containing a point wins; eps_default elsewhere).  lo, hi: npix x 3 pixel
 * corners (x, y, z; dim 1 uses z only, dim 2 x and y); rows: npix x 3 output,
 * the row of the component along cdir (0, 1, 2).  tol, maxeval as in
 * structure(); maxeval == 0 gives the unaveraged 1 / eps at the pixel centre.
 * Host pointers; no mfd_sim needed. */
typedef struct {
  int kind; /* 0 block (axis-aligned), 1 sphere, 2 cylinder */
  double center[3];
  double size[3];  /* block edge lengths */
  double radius;   /* sphere, cylinder */
  double height;   /* cylinder */
  double axis[3];  /* cylinder axis (unit vector) */
  double eps;      /* chi1p1 inside the object */
} mfd_object;
int mfd_subpixel_rows(int dim, int cdir, int64_t npix, const double *lo, const double *hi, double tol, int maxeval,
                      int nobj, const mfd_object *objs, double eps_default, double *rows);

/* Allocation-free flux reduction.  No counterpart in the reference: it is the
 * reduction of mfd_flux (sum_k Re(E conj H) per frequency) for callers that
 * must not allocate device memory when they call it -- hosts whose device
 * memory belongs to another allocator (a framework's caching pool, an FFI
 * host that hands out pre-allocated buffers), loops that cannot take the
 * device synchronisation of cudaMalloc/cudaFree.  Inputs are
 * device pointers to two DFT sum arrays laid out as this engine keeps them
 * (npts * nfreq complex doubles, point-major, i.e. mfd_get_dft's layout), the
 * output a device pointer to nfreq doubles; `stream` is a cudaStream_t (NULL
 * = default stream).  Scratch is a fixed 2 MiB file-scope device array
 * (MFD_NOALLOC_MAX_PARTS rows of MFD_NOALLOC_MAX_FREQ doubles) shared by every
 * call on a device: nfreq above MFD_NOALLOC_MAX_FREQ is rejected, and calls
 * that overlap on the GPU race on it.  The first call on a device looks up the
 * array's address (cudaGetSymbolAddress) with that device current and keeps
 * it; make that first call before any stream capture.  The address belongs
 * to the device's context: after cudaDeviceReset the library must be
 * reloaded before it is called again.  Errors: mfd_noalloc_last_error(). */
#define MFD_NOALLOC_MAX_FREQ 1024
#define MFD_NOALLOC_MAX_PARTS 256
int mfd_flux_noalloc(const double *dft_E, const double *dft_H, int64_t npts, int nfreq, double *flux_out,
                     void *stream);
const char *mfd_noalloc_last_error(void);

/* Number of kernel launches issued by this handle so far (for accounting). */
int64_t mfd_kernel_launches(const mfd_sim *sim);

/* Device-side timing of the last mfd_step call, milliseconds (CUDA events;
 * waits for that call's steps), -1 when the wait fails. */
double mfd_last_step_ms(const mfd_sim *sim);

#ifdef __cplusplus
}
#endif
#endif
