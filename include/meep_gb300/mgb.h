/* C interface of the meep:: drop-in for the Python Simulation front end.
 *
 * The reference's Python layer (python/simulation.py, python/geom.py,
 * python/source.py) drives its C++ core through SWIG: it builds a grid_volume
 * and a structure from a libctl geometry (src/meepgeom.cpp), adds volume
 * sources, DFT flux and DFT field monitors, and steps the fields.  These
 * entry points expose the same C++ calls of this repository's drop-in
 * (include/meep_gb300/meep.hpp) to ctypes, with the geometry evaluated in C++
 * (blocks, spheres, cylinders; later objects take precedence, as in libctl).
 * Cell walls are metallic unless mgb_use_bloch makes them periodic.
 * All functions return 0 on success and -1 on error; mgb_last_error() then
 * holds "meep: ...".
 */
#ifndef MGB_H_
#define MGB_H_

#ifdef __cplusplus
extern "C" {
#endif

#define MGB_MAX_SUS 8

typedef struct mgb_sim mgb_sim;

typedef struct {
  int kind; /* 0 block (axis-aligned), 1 sphere, 2 cylinder */
  double center[3];
  double size[3];  /* block edge lengths */
  double radius;   /* sphere, cylinder */
  double height;   /* cylinder */
  double axis[3];  /* cylinder axis (unit vector) */
  int material;    /* index into the medium table */
} mgb_object;

typedef struct {
  double eps[3];    /* epsilon_diag */
  double d_cond[3]; /* D_conductivity_diag */
  int nsus;
  int sus[MGB_MAX_SUS];          /* indices into the susceptibility table */
  double sigma[MGB_MAX_SUS][3];  /* sigma_diag of each */
} mgb_medium;

typedef struct {
  double frequency, gamma;
  int drude;
} mgb_susceptibility;

/* grid and structure: vol1d/vol2d/vol3d(cell, resolution) centred on the
 * origin; pml: npml rows of (thickness, direction or -1 for all, side
 * (0 high, 1 low) or -1 for both, R_asymptotic, mean_stretch).
 * eps_averaging: subpixel averaging of the permittivity (isotropic media),
 * computed on the GPU by the reference's default material-function method
 * (sphere-quadrature normal, sampled means of eps and 1/eps; tolerance
 * subpixel_tol, at most subpixel_maxeval evaluations per pixel). */
int mgb_create(int dim, const double cell[3], double resolution, double courant, int npml, const double *pml,
               int nmed, const mgb_medium *media, int default_medium, int nobj, const mgb_object *objects,
               int nsus, const mgb_susceptibility *sus, int eps_averaging, double subpixel_tol,
               int subpixel_maxeval, mgb_sim **out);
void mgb_destroy(mgb_sim *s);
const char *mgb_last_error(void);

/* sources: kind 0 gaussian_src_time(p0 = frequency, p1 = width, p2 = start
 * time, p3 = end time); kind 1 continuous_src_time(p0 = frequency, p1 =
 * width, p2 = start time, p3 = end time, p4 = slowness).  Added with
 * fields::add_volume_source(component, src, volume(center, size), amp). */
int mgb_add_source(mgb_sim *s, int component, int kind, const double *params, int is_integrated,
                   const double center[3], const double size[3], double amp_re, double amp_im);
double mgb_last_source_time(const mgb_sim *s);

/* flux: nreg rows of (center[3], size[3], direction or -1 for the normal of
 * the region, weight); freqs[nfreq]; returns a handle */
int mgb_add_flux(mgb_sim *s, int nreg, const double *regions, int nfreq, const double *freqs, int decimation,
                 int *handle);
int mgb_flux(mgb_sim *s, int handle, double *out);
/* the DFT sums of a flux's E (part 0) or H (part 1) chunks as one array of
 * *n complex values (re/im); out NULL gives only *n.  load replaces them
 * (n must match); scale multiplies both (dft_flux::scale_dfts) */
int mgb_flux_data(mgb_sim *s, int handle, int part, double *out, size_t *n);
int mgb_load_flux_data(mgb_sim *s, int handle, int part, const double *in, size_t n);
int mgb_flux_scale(mgb_sim *s, int handle, double re, double im);
/* the same for any DFT object: kind 0 flux (parts E, H), 1 force (offdiag1,
 * offdiag2, diag), 2 near2far (F), 3 energy (E, D, H, B) */
int mgb_dft_data(mgb_sim *s, int kind, int handle, int part, double *out, size_t *n);
int mgb_load_dft_data(mgb_sim *s, int kind, int handle, int part, const double *in, size_t n);
int mgb_scale_dft_data(mgb_sim *s, int kind, int handle, int part, double re, double im);
/* local density of states (dft_ldos): create, update before every step and
 * after the last (the dft_ldos step function), then ldos[nfreq] and the
 * DFTs F, J (nfreq complex, re/im) */
int mgb_ldos_create(mgb_sim *s, int nfreq, const double *freqs, int *handle);
int mgb_ldos_update(mgb_sim *s, int handle);
int mgb_ldos_results(mgb_sim *s, int handle, double *ldos, double *F, double *J);
/* energy spectra (fields::add_dft_energy) over regions as for mgb_add_flux;
 * mgb_energy: which 0 electric, 1 magnetic, 2 total, nfreq values */
int mgb_add_energy(mgb_sim *s, int nreg, const double *regions, int nfreq, const double *freqs, int decimation,
                   int *handle);
int mgb_energy(mgb_sim *s, int handle, int which, double *out);
/* Maxwell-stress force (fields::add_dft_force): regions as for mgb_add_flux,
 * direction = the force's direction; mgb_force gives nfreq values */
int mgb_add_force(mgb_sim *s, int nreg, const double *regions, int nfreq, const double *freqs, int decimation,
                  int *handle);
int mgb_force(mgb_sim *s, int handle, double *out);
/* near-to-far surfaces: regions as for mgb_add_flux; nperiods > 1 sums
 * lattice images along periodic directions (fields::add_dft_near2far) */
int mgb_add_near2far(mgb_sim *s, int nreg, const double *regions, int nfreq, const double *freqs, int decimation,
                     int nperiods, int *handle);
/* far fields at npts points xyz[3 npts]: out[npts * nfreq * 6 * 2], point
 * slowest, then frequency, then Ex..Hz, re/im interleaved */
int mgb_near2far_points(mgb_sim *s, int handle, int npts, const double *xyz, double *out);
/* get_farfields_array over volume(center, size) at `resolution`: with out
 * NULL only dims[0..2] (points per direction, 1 for absent ones) and *rank;
 * else out receives 12 * N * nfreq doubles in the reference's layout
 * ((component * 2 + re/im) * N + point) * nfreq + frequency */
int mgb_near2far_array(mgb_sim *s, int handle, const double center[3], const double size[3], double resolution,
                       double *out, int dims[3], int *rank);
/* dft_near2far::flux through volume(center, size) with normal `direction` */
int mgb_near2far_flux(mgb_sim *s, int handle, int direction, const double center[3], const double size[3],
                      double resolution, double *out);
/* dft_near2far::scale_dfts */
int mgb_near2far_scale(mgb_sim *s, int handle, double re, double im);
/* the homogeneous medium seen by the surfaces */
int mgb_near2far_medium(mgb_sim *s, int handle, double *eps, double *mu);
/* DFT fields of ncomp components over volume(center, size) */
int mgb_add_dft_fields(mgb_sim *s, int ncomp, const int *components, const double center[3],
                       const double size[3], int nfreq, const double *freqs, int yee_grid, int decimation,
                       int *handle);
/* shape[3] (points per direction, 1 for absent ones) of component c of a DFT
 * fields handle; out (may be NULL) receives shape product complex values of
 * frequency ifreq, interleaved re/im, last direction fastest */
int mgb_dft_fields_array(mgb_sim *s, int handle, int component, int ifreq, double *out, int shape[3]);

int mgb_step(mgb_sim *s, int n);
int mgb_time(const mgb_sim *s, double *time, double *round_time, double *dt, int *t);
/* fields::get_field at n points (interpolated as the reference does) */
int mgb_get_field_points(mgb_sim *s, int component, int n, const double *xyz, double *re, double *im);
/* component c at every Yee point of the cell, x slowest (n = prod(N_d + 1)
 * values; out NULL returns the count in *n); part 0 real, 1 imaginary */
int mgb_yee_array(mgb_sim *s, int component, int part, double *out, long long *n);
/* Bloch-periodic boundaries in every direction of the cell with wavevector
 * k (fields::use_bloch(vec)); before the first step.  A nonzero k makes the
 * fields complex. */
int mgb_use_bloch(mgb_sim *s, const double k[3]);
/* A material grid over the block (center, size): weights n[0] x n[1] x n[2]
 * (row-major), projection (beta, eta), eps = eps1 + p (eps2 - eps1) per
 * direction (structure::add_material_grid); right after mgb_create. */
int mgb_add_material_grid(mgb_sim *s, const double center[3], const double size[3], const int n[3],
                          const double *weights, double beta, double eta, const double eps1[3],
                          const double eps2[3]);
/* epsilon of the material at n points (no averaging) */
int mgb_get_epsilon_points(mgb_sim *s, int n, const double *xyz, double *eps);

#ifdef __cplusplus
}
#endif
#endif
