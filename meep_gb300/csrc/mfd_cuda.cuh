// CUDA backend of the FDTD stepping engine, templated on the field precision R
// (double or float).  Instantiated by mfd_cuda_f64.cu and mfd_cuda_f32.cu.
//
// Data layout in HBM: one array per field component over the whole cell
// (Plan::nstore points, last direction unit-stride and padded to a multiple of
// 8 points), auxiliary PML/conductivity arrays of the same shape, 1-D PML
// coefficient tables per direction indexed by half-pixel position.  Every
// kernel advances the points of one component inside a box of point indices;
// the reference's per-chunk choice of formula is recomputed per point from its
// chunk region (see mfd_plan.hpp), so no halo exchange exists.
//
// Per-point arithmetic follows, in the same operation order:
//   curl            step_curl               src/step_generic.cpp:65-249
//   E/H update      step_update_EDHB        src/step_generic.cpp:566-785
//   polarisation    lorentzian update_P     src/susceptibility.cpp:188-262
//   sources         step_source             src/step.cpp:295-318,
//                   integrated sources      src/update_eh.cpp:126-136
//   DFT             dft_chunk::update_dft   src/dft.cpp:266-308
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "mfd_backend.hpp"
#include "mfd_near2far.hpp"

namespace mfd {
namespace cuda_impl {

static const double kPi = 3.141592653589793238462643383276;

inline void cuda_check(cudaError_t e, const char *what) {
  if (e != cudaSuccess)
    throw Error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

// Region geometry shared by all kernels (passed by value).
struct Geo {
  int N[3];
  int T[3][2];
  int pml[3];        // PML exists along direction
  long long stride[3];
  int fast, mid, slow; // direction mapped to grid x / y / z
};

__device__ __forceinline__ int region_of(const Geo &g, int d, int pos) {
  if (g.T[d][0] > 0 && pos <= 2 * g.T[d][0]) return 0;
  if (g.T[d][1] > 0 && pos > 2 * (g.N[d] - g.T[d][1])) return 2;
  return 1;
}
__device__ __forceinline__ bool slab(const Geo &g, int d, int pos) {
  return g.pml[d] && region_of(g, d, pos) != 1;
}

struct Box {
  int lo[3], n[3];
};

// point indices of this thread inside the box; false if outside
__device__ __forceinline__ bool box_point(const Geo &g, const Box &b, int k[3]) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  int m = blockIdx.y * blockDim.y + threadIdx.y;
  int s = blockIdx.z;
  if (a >= b.n[g.fast] || m >= b.n[g.mid] || s >= b.n[g.slow]) return false;
  k[g.fast] = b.lo[g.fast] + a;
  k[g.mid] = b.lo[g.mid] + m;
  k[g.slow] = b.lo[g.slow] + s;
  return true;
}

__device__ __forceinline__ long long lin(const Geo &g, const int k[3]) {
  return k[0] * g.stride[0] + k[1] * g.stride[1] + k[2] * g.stride[2];
}

template <typename R> struct Tables {
  const R *sig[3], *kap[3], *siginv[3];
};

// ------------------------------------------------------------------ curl
template <typename R> struct CurlArgs {
  R *f, *fu, *fcnd;
  const R *cnd, *cndinv;
  const R *g1, *g1h, *g2, *g2h; // g*h: H arrays for D curls (null for B curls)
  int g1dir, g2dir;
  long long s1, s2;
  R dtdx, dt2;
  int dsig, dsigu;
  int shift[3];
  unsigned cond_chunks; // bit r: chunk region r (rx*9+ry*3+rz) has conductivity
  Box box;
};

template <typename R>
__global__ void __launch_bounds__(256) curl_kernel(Geo g, Tables<R> tb, CurlArgs<R> a) {
  int k[3];
  if (!box_point(g, a.box, k)) return;
  const long long i = lin(g, k);
  const R *G1 = a.g1;
  if (a.g1h && slab(g, a.g1dir, 2 * k[a.g1dir])) G1 = a.g1h;
  R X = G1[i + a.s1] - G1[i];
  if (a.g2) {
    const R *G2 = a.g2;
    if (a.g2h && slab(g, a.g2dir, 2 * k[a.g2dir])) G2 = a.g2h;
    X = X + G2[i] - G2[i + a.s2];
  }
  const bool sg = a.dsig >= 0 && slab(g, a.dsig, a.shift[a.dsig] + 2 * k[a.dsig]);
  const bool su = a.dsigu >= 0 && slab(g, a.dsigu, a.shift[a.dsigu] + 2 * k[a.dsigu]);
  bool hc = a.cnd != nullptr;
  if (sg && hc) {
    int r = region_of(g, 0, a.shift[0] + 2 * k[0]) * 9 + region_of(g, 1, a.shift[1] + 2 * k[1]) * 3 +
            region_of(g, 2, a.shift[2] + 2 * k[2]);
    hc = (a.cond_chunks >> r) & 1u;
  }
  R *F = a.f;
  const R one = R(1);
  if (!sg) {
    if (!su) {
      if (hc) F[i] = ((one - a.dt2 * a.cnd[i]) * F[i] - a.dtdx * X) * a.cndinv[i];
      else F[i] -= a.dtdx * X;
    }
    else {
      const int ku = a.shift[a.dsigu] + 2 * k[a.dsigu];
      R fprev = a.fu[i];
      R fun;
      if (hc) fun = ((one - a.dt2 * a.cnd[i]) * fprev - a.dtdx * X) * a.cndinv[i];
      else fun = fprev - a.dtdx * X;
      a.fu[i] = fun;
      F[i] = tb.siginv[a.dsigu][ku] * ((tb.kap[a.dsigu][ku] - tb.sig[a.dsigu][ku]) * F[i] + fun - fprev);
    }
  }
  else {
    const int kk = a.shift[a.dsig] + 2 * k[a.dsig];
    const R ks = tb.kap[a.dsig][kk] - tb.sig[a.dsig][kk], si = tb.siginv[a.dsig][kk];
    if (!su) {
      if (hc) {
        R fcp = a.fcnd[i];
        R fcn = ((one - a.dt2 * a.cnd[i]) * fcp - a.dtdx * X) * a.cndinv[i];
        a.fcnd[i] = fcn;
        F[i] = (ks * F[i] + (fcn - fcp)) * si;
      }
      else
        F[i] = (ks * F[i] - a.dtdx * X) * si;
    }
    else {
      const int ku = a.shift[a.dsigu] + 2 * k[a.dsigu];
      R fprev = a.fu[i];
      R fun;
      if (hc) {
        R fcp = a.fcnd[i];
        R fcn = ((one - a.dt2 * a.cnd[i]) * fcp - a.dtdx * X) * a.cndinv[i];
        a.fcnd[i] = fcn;
        fun = (ks * fprev + (fcn - fcp)) * si;
      }
      else
        fun = (ks * fprev - a.dtdx * X) * si;
      a.fu[i] = fun;
      F[i] = tb.siginv[a.dsigu][ku] * ((tb.kap[a.dsigu][ku] - tb.sig[a.dsigu][ku]) * F[i] + fun - fprev);
    }
  }
}

// ------------------------------------------------- H = B in the PML slab
template <typename R> struct HArgs {
  R *h, *fw;
  const R *b;
  int dir;
  int shift[3];
  Box box;
};

template <typename R> __global__ void __launch_bounds__(256) h_pml_kernel(Geo g, Tables<R> tb, HArgs<R> a) {
  int k[3];
  if (!box_point(g, a.box, k)) return;
  const int kw = a.shift[a.dir] + 2 * k[a.dir];
  if (!slab(g, a.dir, kw)) return;
  const long long i = lin(g, k);
  R fwprev = a.fw[i], kapwkw = tb.kap[a.dir][kw], sigwkw = tb.sig[a.dir][kw];
  R fwn = a.b[i];
  a.fw[i] = fwn;
  a.h[i] += (kapwkw + sigwkw) * fwn - (kapwkw - sigwkw) * fwprev;
}

// --------------------------------------------------- E, then its poles
template <typename R> struct PoleArgs {
  R *P, *PP;
  const R *s;
  R gamma1inv, gamma1, w0, w0d;
};

template <typename R> struct EArgs {
  R *e, *fw;
  const R *dfield, *chi;
  int dir;
  int shift[3];
  int npoles;
  PoleArgs<R> pole[MAX_POLES];
  Box box;
  // dfield already holds D - P - integrated sources (off-diagonal update:
  // f_minus_p of every D component is formed before any E is computed)
  int pre;
  // off-diagonal terms: D component g[q] along direction with stride so[q],
  // weights u[q]; s = stride along dir
  int noff;
  const R *og[2], *ou[2];
  long long so[2], s;
};

template <typename R> struct EPoint {
  R e, fw;
  R p[MAX_POLES], pp[MAX_POLES];
};

// Computes the new E (and f_w, P, P_prev) of one point; srcA is subtracted
// from D - P (integrated sources), nsrc == 0 for ordinary points.
template <typename R>
__device__ __forceinline__ void e_point(const Geo &g, const Tables<R> &tb, const EArgs<R> &a,
                                        const int k[3], long long i, int nsrc, const R *srcA,
                                        EPoint<R> &out) {
  R gs = a.dfield[i];
  if (!a.pre)
    for (int q = 0; q < a.npoles; q++)
      if (a.pole[q].P) gs -= a.pole[q].P[i];
  for (int j = 0; j < nsrc; j++)
    gs -= srcA[j];
  const R us = a.chi[i];
  R val = (gs * us);
  // OFFDIAG(u, g, sx) = 0.25 ((g[i] + g[i-sx]) u[i] + (g[i+s] + g[i+s-sx]) u[i+s])
  // (src/step_generic.cpp:580-582)
  for (int q = 0; q < a.noff; q++) {
    const R *og = a.og[q], *ou = a.ou[q];
    const long long sx = a.so[q], s = a.s;
    val = val + R(0.25) * ((og[i] + og[i - sx]) * ou[i] + (og[i + s] + og[(i + s) - sx]) * ou[i + s]);
  }
  const int kw = a.shift[a.dir] + 2 * k[a.dir];
  const bool w = slab(g, a.dir, kw);
  R W;
  if (w) {
    R fwprev = a.fw[i], kapwkw = tb.kap[a.dir][kw], sigwkw = tb.sig[a.dir][kw];
    R fwn = val;
    out.fw = fwn;
    out.e = a.e[i] + ((kapwkw + sigwkw) * fwn - (kapwkw - sigwkw) * fwprev);
    W = fwn;
  }
  else {
    out.e = val;
    out.fw = R(0);
    W = out.e;
  }
  for (int q = 0; q < a.npoles; q++) {
    const PoleArgs<R> &pl = a.pole[q];
    if (!pl.P) continue;
    R pcur = pl.P[i];
    out.p[q] = pl.gamma1inv * (pcur * (R(2) - pl.w0d) - pl.gamma1 * pl.PP[i] + pl.w0 * (pl.s[i] * W));
    out.pp[q] = pcur;
  }
}

template <typename R>
__device__ __forceinline__ void e_store(const Geo &g, const EArgs<R> &a, const int k[3], long long i,
                                        const EPoint<R> &v) {
  a.e[i] = v.e;
  if (slab(g, a.dir, a.shift[a.dir] + 2 * k[a.dir])) a.fw[i] = v.fw;
  for (int q = 0; q < a.npoles; q++)
    if (a.pole[q].P) {
      a.pole[q].P[i] = v.p[q];
      a.pole[q].PP[i] = v.pp[q];
    }
}

template <typename R> __global__ void __launch_bounds__(256) e_kernel(Geo g, Tables<R> tb, EArgs<R> a) {
  int k[3];
  if (!box_point(g, a.box, k)) return;
  const long long i = lin(g, k);
  EPoint<R> v;
  e_point(g, tb, a, k, i, 0, (const R *)nullptr, v);
  e_store(g, a, k, i, v);
}

// ----------------------------------------- integrated E sources (sparse)
// One entry per distinct source point of one E component: up to MAXS source
// terms, each amp * dipole(src) with the dipole passed per step.
constexpr int MAXS = 4;
struct SrcPoint {
  long long i;          // storage index
  int k[3];
  int nterm;
  int src[MAXS];
  double amp[MAXS][2];
};

// Empty kernel put on the main stream between a join and the next fork when
// no other kernel sits there: with the fork's event recorded right behind the
// join's waits, the next half-step's launches started about 6 us later on
// GB300 (measured over the 256^3 and 384^2 x 192 steps)
static __global__ void stream_order_kernel() {}

template <typename R> struct SrcBuf {
  EPoint<R> *v;
};

struct DipoleVals {
  double re[16], im[16];
};

// term t of a source point: the real part of amp * dipole (the std::complex
// product), rounded product by product as on the host
__device__ __forceinline__ double src_term(const SrcPoint &sp, int t, const DipoleVals &dv) {
  return __dsub_rn(__dmul_rn(sp.amp[t][0], dv.re[sp.src[t]]), __dmul_rn(sp.amp[t][1], dv.im[sp.src[t]]));
}

// Integrated E sources at points without an active pole and outside the E
// slab of their own direction, after the D/E launches left D final there
// and E = D chi1inv: E = (D - the terms in list order) chi1inv, the f_minus_p
// of update_eh less the sources (src/update_eh.cpp:108-137; a pole with zero
// sigma keeps P = 0, and D - 0 = D)
template <typename R>
__global__ void src_e_kernel(R *e, const R *dfield, const R *chi, const SrcPoint *pts, int n, DipoleVals dv) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const SrcPoint &sp = pts[j];
  R gs = dfield[sp.i];
  for (int t = 0; t < sp.nterm; t++)
    gs -= R(src_term(sp, t, dv));
  e[sp.i] = gs * chi[sp.i];
}

template <typename R>
__global__ void src_pre_kernel(Geo g, Tables<R> tb, EArgs<R> a, const SrcPoint *pts, int n,
                               DipoleVals dv, EPoint<R> *out) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const SrcPoint &sp = pts[j];
  R A[MAXS];
  for (int t = 0; t < sp.nterm; t++)
    A[t] = R(src_term(sp, t, dv));
  e_point(g, tb, a, sp.k, sp.i, sp.nterm, A, out[j]);
}

// f_minus_p of one D component over the whole storage: D minus the
// polarizations in list order (src/update_eh.cpp:108-123, subtract_P
// src/susceptibility.cpp:264-279); used by the off-diagonal E update, which
// reads D - P of the other components at neighbouring points
template <typename R> struct FmpArgs {
  R *out;
  const R *d;
  const R *p[MAX_POLES];
  int np;
  long long n;
};

template <typename R> __global__ void fmp_kernel(FmpArgs<R> a) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  R v = a.d[i];
  for (int q = 0; q < a.np; q++)
    if (a.p[q]) v -= a.p[q][i];
  a.out[i] = v;
}

// integrated E sources subtracted from f_minus_p (src/update_eh.cpp:126-137);
// f_minus_p at the source point is formed afresh from D and P first, since a
// source may sit on a point that the D pass does not visit (a wall)
template <typename R> __global__ void src_fmp_kernel(FmpArgs<R> fa, const SrcPoint *pts, int n, DipoleVals dv) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const SrcPoint &sp = pts[j];
  R *fmp = fa.out;
  R v = fa.d[sp.i];
  for (int q = 0; q < fa.np; q++)
    if (fa.p[q]) v -= fa.p[q][sp.i];
  for (int t = 0; t < sp.nterm; t++) {
    const double re = src_term(sp, t, dv);
    v -= R(re);
  }
  fmp[sp.i] = v;
}

template <typename R>
__global__ void src_post_kernel(Geo g, EArgs<R> a, const SrcPoint *pts, int n, const EPoint<R> *in) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  e_store(g, a, pts[j].k, pts[j].i, in[j]);
}

} // namespace cuda_impl
} // namespace mfd
#include "mfd_fused.cuh"
#include "mfd_k3d.cuh"
#include "mfd_q3d.cuh"
#include "mfd_q3f.cuh"
#include "mfd_dft_tc.cuh"
#include "mfd_adjoint.cuh"
#include "mfd_adjoint3.cuh"
#include "mfd_matgrid.cuh"
namespace mfd {
namespace cuda_impl {

// current (non-integrated) sources on D or B: f -= Re(amp*J*dt*condinv)
struct CurPoint {
  long long i;
  int src;
  double amp[2];
};

template <typename R>
__global__ void src_current_kernel(R *f, const R *cndinv, const CurPoint *pts, int n,
                                   DipoleVals cur, double dt) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const CurPoint &p = pts[j];
  // A = amp * current * dt (* condinv), complex arithmetic of the reference
  double cre = cur.re[p.src], cim = cur.im[p.src];
  double are = p.amp[0] * cre - p.amp[1] * cim;
  double aim = p.amp[0] * cim + p.amp[1] * cre;
  are = are * dt;
  aim = aim * dt;
  if (cndinv) {
    double ci = double(cndinv[p.i]);
    are = are * ci;
  }
  (void)aim;
  f[p.i] -= R(are);
}

// ------------------------------------------------------------------ DFT
template <typename R> struct DftArgs {
  const R *f, *fb;   // component array; fb = B array for H components (else null)
  const R *fim, *fbim; // imaginary parts of complex (Bloch) fields, else null
  int hdir;          // direction of the H component (H/B selection)
  int hshift;        // shift of the component along hdir
  const double *w[3];
  double dV;
  int include_weights;
  int sqrt_w; // the square root of the weight product
  int dim;
  int lo[3], n[3];
  int ad0, ad1; // averaging directions (-1 none)
  double2 *acc;
  const double2 *ph;
  int nf;
  long long npts;
};

template <typename R>
__device__ __forceinline__ R dft_val(const Geo &g, const DftArgs<R> &a, const int k[3]) {
  const long long i = lin(g, k);
  if (a.fb && !slab(g, a.hdir, a.hshift + 2 * k[a.hdir])) return a.fb[i];
  return a.f[i];
}

static __global__ void dft_phase_kernel(const double *freq, int nf, double time, double sre, double sim,
                                 double2 *ph) {
  int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nf) return;
  double s, c;
  sincos(2 * kPi * freq[w] * time, &s, &c);
  ph[w] = make_double2(c * sre - s * sim, c * sim + s * sre);
}

// weighted (and centred) field value of monitor point p (update_dft,
// src/dft.cpp:275-295): weight product in the reference's loop order
template <typename R> __device__ __forceinline__ R dft_point_value(const Geo &g, const DftArgs<R> &a, long long p) {
  int q[3];
  q[2] = int(p % a.n[2]);
  long long r = p / a.n[2];
  q[1] = int(r % a.n[1]);
  q[0] = int(r / a.n[1]);
  int k[3] = {a.lo[0] + q[0], a.lo[1] + q[1], a.lo[2] + q[2]};
  double wgt = 1.0;
  if (a.include_weights) {
    double wx = a.w[0] ? a.w[0][q[0]] : 1.0;
    double wy = a.w[1] ? a.w[1][q[1]] : 1.0;
    double wz = a.w[2] ? a.w[2][q[2]] : 1.0;
    if (a.dim == 2) wgt = wy * (wx * (a.dV * 1.0));
    else if (a.dim == 3) wgt = wz * (wy * (a.dV * wx));
    else wgt = 1.0 * (1.0 * (a.dV * wz));
    if (a.sqrt_w) wgt = sqrt(wgt);
  }
  if (a.ad1 >= 0) {
    int k1[3] = {k[0], k[1], k[2]}, k2[3] = {k[0], k[1], k[2]}, k3[3] = {k[0], k[1], k[2]};
    k1[a.ad0]++;
    k2[a.ad1]++;
    k3[a.ad0]++;
    k3[a.ad1]++;
    return R((wgt * 0.25) * (dft_val(g, a, k) + dft_val(g, a, k1) + dft_val(g, a, k2) + dft_val(g, a, k3)));
  }
  if (a.ad0 >= 0) {
    int k1[3] = {k[0], k[1], k[2]};
    k1[a.ad0]++;
    return R((wgt * 0.5) * (dft_val(g, a, k) + dft_val(g, a, k1)));
  }
  return R(wgt * dft_val(g, a, k));
}

// direct accumulation, one thread per (point, frequency): the FP64 path
template <typename R> __global__ void dft_kernel(Geo g, DftArgs<R> a) {
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  long long total = a.npts * a.nf;
  if (t >= total) return;
  long long p = t / a.nf;
  int w = int(t - p * a.nf);
  const R fv = dft_point_value(g, a, p);
  double2 ph = a.ph[w];
  double2 acc = a.acc[t];
  if (a.fim) {
    // complex fields: acc += phase * (f_re + i f_im) (src/dft.cpp:296-299)
    DftArgs<R> ai = a;
    ai.f = a.fim;
    ai.fb = a.fbim;
    const double fr = double(fv), fi = double(dft_point_value(g, ai, p));
    acc.x += ph.x * fr - ph.y * fi;
    acc.y += ph.x * fi + ph.y * fr;
  }
  else {
    acc.x += double(fv) * ph.x;
    acc.y += double(fv) * ph.y;
  }
  a.acc[t] = acc;
}

// Bloch-periodic ghost plane along direction d: dst = phase * src for the two
// parts (complex<realnum> product, src/step.cpp:186-192); im may be null for
// real fields (phase then +-1)
template <typename R>
__global__ void ghost_plane_kernel(R *re, R *im, long long dst, long long src, int n1, int n2, long long s1,
                                   long long s2, R pr, R pi) {
  const int j2 = blockIdx.x * blockDim.x + threadIdx.x, j1 = blockIdx.y;
  if (j2 >= n2 || j1 >= n1) return;
  const long long o = j1 * s1 + j2 * s2;
  const R vr = re[src + o];
  if (im) {
    const R vi = im[src + o];
    re[dst + o] = pr * vr - pi * vi;
    im[dst + o] = pr * vi + pi * vr;
  }
  else
    re[dst + o] = pr * vr;
}

// Blocked DFT (FP32 path): each sampled step stores the monitor values in one
// row of a [T][npts] buffer; every T samples the block is contracted against
// the [T][2 nfreq] phase matrix (phases generated in FP64 from the exact sample
// times, so nothing drifts between blocks) with FP32 products and FP32 sums of
// T terms, and the block result is added to the FP64 running sums.
constexpr int DFT_BLOCK_T = 64;

template <typename R> __global__ void dft_sample_kernel(Geo g, DftArgs<R> a, float *row) {
  long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= a.npts) return;
  row[p] = float(dft_point_value(g, a, p));
}

// phase matrix B[t][w] = polar(1, 2 pi f_w time_t) * scale, times of the block's
// samples time_t = (tn0 + t dec) dt (- dt/2 for H and B)
static __global__ void dft_block_phase_kernel(const double *freq, int nf, int cnt, long long tn0, int dec,
                                              double dt, int half, double sre, double sim, float2 *B) {
  int t = blockIdx.y;
  int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nf || t >= cnt) return;
  double timeE = (tn0 + (long long)t * dec) * dt;
  double time = half ? timeE - 0.5 * dt : timeE;
  double s, c;
  sincos(2 * kPi * freq[w] * time, &s, &c);
  B[(long long)t * nf + w] = make_float2(float(c * sre - s * sim), float(c * sim + s * sre));
}

static __global__ void __launch_bounds__(128) dft_contract_kernel(const float *A, int cnt, long long npts,
                                                                   const float2 *B, int nf, double2 *acc) {
  extern __shared__ float2 sB[]; // [cnt][chunk]
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  float a[DFT_BLOCK_T];
#pragma unroll
  for (int t = 0; t < DFT_BLOCK_T; t++)
    a[t] = (t < cnt && p < npts) ? A[(long long)t * npts + p] : 0.0f;
  const int chunk = 64;
  for (int w0 = 0; w0 < nf; w0 += chunk) {
    const int wn = min(chunk, nf - w0);
    __syncthreads();
    for (int q = threadIdx.x; q < cnt * wn; q += blockDim.x) {
      const int t = q / wn, w = q - t * wn;
      sB[t * chunk + w] = B[(long long)t * nf + w0 + w];
    }
    __syncthreads();
    if (p < npts)
      for (int w = 0; w < wn; w++) {
        float sr = 0.f, si = 0.f;
#pragma unroll
        for (int t = 0; t < DFT_BLOCK_T; t++)
          if (t < cnt) {
            const float2 b = sB[t * chunk + w];
            sr = fmaf(a[t], b.x, sr);
            si = fmaf(a[t], b.y, si);
          }
        double2 v = acc[p * nf + w0 + w];
        v.x += double(sr);
        v.y += double(si);
        acc[p * nf + w0 + w] = v;
      }
  }
}

// flux: sum_k Re(E conj H) per frequency, in double (FP64 units are scarce on
// this part, so the reduction is a plain deterministic tree, no compensation).
// Threads of a warp take consecutive frequencies of one point (coalesced rows
// of the [npts][nf] sums); the 8 warps of a block stride over points; block
// partials go to a buffer that a second kernel reduces in a fixed order.
static __global__ void flux_partial_kernel(const double2 *E, const double2 *H, long long npts, int nf,
                                           double *partial) {
  const int w = blockIdx.x * 32 + threadIdx.x;
  double s = 0.0;
  if (w < nf)
    for (long long k = blockIdx.y * 8 + threadIdx.y; k < npts; k += 8LL * gridDim.y) {
      const double2 e = E[k * nf + w], h = H[k * nf + w];
      s += e.x * h.x + e.y * h.y;
    }
  __shared__ double red[8][33];
  red[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && w < nf) {
    double t = red[0][threadIdx.x];
    for (int r = 1; r < 8; r++)
      t += red[r][threadIdx.x];
    partial[(long long)blockIdx.y * nf + w] = t;
  }
}

// out[w] (+)= sum over the partials of frequency w: 32 frequencies x 8 lanes
// per block, tree over the lanes
static __global__ void flux_final_kernel(const double *partial, int nparts, int nf, double *out, int accumulate) {
  const int w = blockIdx.x * 32 + threadIdx.x;
  double s = 0.0;
  if (w < nf)
    for (int q = threadIdx.y; q < nparts; q += 8)
      s += partial[(long long)q * nf + w];
  __shared__ double red[8][33];
  red[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && w < nf) {
    double t = red[0][threadIdx.x];
    for (int r = 1; r < 8; r++)
      t += red[r][threadIdx.x];
    out[w] = accumulate ? out[w] + t : t;
  }
}

// Divergence test of fields::step() (src/step.cpp:137-138): half the sum of
// Re(conj(E_d) D_d) with both interpolated at the cell centre
// (Plan::center_probe); a non-finite value sets a flag in host-mapped
// memory, which the host reads without a copy in the stream.
template <typename R> struct FiniteProbe {
  const R *e[3], *d[3], *ei[3], *di[3];
  int n[3];
  long long idx[3][8];
  double w[3][8];
  int *flag;
};
template <typename R> __global__ void finite_probe_kernel(const FiniteProbe<R> p) {
  double sum = 0.0;
  for (int c = 0; c < 3; c++) {
    if (!p.e[c]) continue;
    double er = 0, dr = 0, ei = 0, di = 0;
    for (int j = 0; j < p.n[c]; j++) {
      const long long i = p.idx[c][j];
      er += p.w[c][j] * double(p.e[c][i]);
      dr += p.w[c][j] * double(p.d[c][i]);
      if (p.ei[c]) {
        ei += p.w[c][j] * double(p.ei[c][i]);
        di += p.w[c][j] * double(p.di[c][i]);
      }
    }
    sum += er * dr + ei * di;
  }
  if (!isfinite(sum * 0.5)) {
    *(volatile int *)p.flag = 1;
    __threadfence_system();
  }
}

// ---------------------------------------------------------------- backend
template <typename R> class CudaBackend : public Backend {
public:
  explicit CudaBackend(const Plan &p) {
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream");
    cuda_check(cudaEventCreate(&ev0), "event");
    cuda_check(cudaEventCreate(&ev1), "event");
    // the side streams carry the PML shell of each half-step: higher priority,
    // so their (latency-bound) blocks are dispatched ahead of the pending
    // core blocks and finish under them instead of trailing after them
    int prio_lo = 0, prio_hi = 0;
    cuda_check(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi), "stream priorities");
    for (int q = 0; q < NSIDE; q++) {
      cuda_check(cudaStreamCreateWithPriority(&side[q], cudaStreamNonBlocking, prio_hi), "stream");
      cuda_check(cudaEventCreateWithFlags(&side_ev[q], cudaEventDisableTiming), "event");
    }
    cuda_check(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming), "event");
    // E/D monitors of the 3-D step: samples and block contractions on
    // low-priority streams, their blocks filling in beside the next B
    // half-step (high priority measured 2 us per step slower)
    cuda_check(cudaStreamCreateWithPriority(&dstream, cudaStreamNonBlocking, prio_lo), "stream");
    cuda_check(cudaStreamCreateWithPriority(&fstream, cudaStreamNonBlocking, prio_lo), "stream");
    for (cudaEvent_t *e : {&dft_in_ev, &dft_out_ev, &fl_in_ev, &fl_out_ev})
      cuda_check(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "event");
    (void)p;
  }
  ~CudaBackend() override {
    for (void *ptr : allocs)
      cudaFree(ptr);
    if (h_nonfinite) cudaFreeHost(h_nonfinite);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    for (int q = 0; q < NSIDE; q++) {
      cudaEventDestroy(side_ev[q]);
      cudaStreamDestroy(side[q]);
    }
    cudaEventDestroy(fork_ev);
    for (DMon &dm : mons)
      for (cudaEvent_t e : dm.fdone)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : {dft_in_ev, dft_out_ev, fl_in_ev, fl_out_ev})
      cudaEventDestroy(e);
    if (sgexec) cudaGraphExecDestroy(sgexec);
    if (sgraph) cudaGraphDestroy(sgraph);
    cudaStreamDestroy(dstream);
    cudaStreamDestroy(fstream);
    cudaStreamDestroy(stream);
  }

  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // side streams: the launches of one half-step touch disjoint points, so
  // they run side by side (filling each other's tail waves) and join the main
  // stream before the next half-step
  static constexpr int NSIDE = 6;
  cudaStream_t side[NSIDE] = {};
  cudaEvent_t side_ev[NSIDE] = {}, fork_ev = nullptr;
  // fork: the point of the main stream that side streams start from; S(q):
  // side stream q, made to wait for that point on its first use; join: the
  // main stream waits for the side streams used since the fork (every
  // wait costs: the FP32 step measured 2-3 us faster with three side
  // streams joined instead of six)
  cudaEvent_t fork_cur = nullptr;
  unsigned side_used = 0;
  void fork() {
    if (fork_from) fork_cur = fork_from;
    else {
      cuda_check(cudaEventRecord(fork_ev, stream), "event record");
      fork_cur = fork_ev;
    }
    fork_from = nullptr;
    side_used = 0;
  }
  cudaStream_t S(int q) {
    if (!((side_used >> q) & 1u)) {
      cuda_check(cudaStreamWaitEvent(side[q], fork_cur, 0), "stream wait");
      side_used |= 1u << q;
    }
    return side[q];
  }
  void join() {
    for (int q = 0; q < NSIDE; q++)
      if ((side_used >> q) & 1u) {
        cuda_check(cudaEventRecord(side_ev[q], side[q]), "event record");
        cuda_check(cudaStreamWaitEvent(stream, side_ev[q], 0), "stream wait");
      }
    side_used = 0;
  }
  // DFT work off the main stream: the samples of E/D monitors (read E or D
  // after a step; the next B half-step runs beside them, the next D/E
  // half-step waits for them) and the block contractions (read the staged
  // samples, write the running sums; everything else that reads the sums or
  // the fields waits for both first)
  cudaStream_t dstream = nullptr, fstream = nullptr;
  cudaEvent_t dft_in_ev = nullptr, dft_out_ev = nullptr, fl_in_ev = nullptr, fl_out_ev = nullptr;
  cudaEvent_t fork_from = nullptr; // event at the main stream's tail for the next fork, if any
  bool dft_pending = false, fl_pending = false;
  void join_samples() {
    fork_from = nullptr;
    if (!dft_pending) return;
    cuda_check(cudaEventRecord(dft_out_ev, dstream), "event record");
    cuda_check(cudaStreamWaitEvent(stream, dft_out_ev, 0), "stream wait");
    dft_pending = false;
  }
  void join_dft() {
    join_samples();
    if (!fl_pending) return;
    cuda_check(cudaEventRecord(fl_out_ev, fstream), "event record");
    cuda_check(cudaStreamWaitEvent(stream, fl_out_ev, 0), "stream wait");
    fl_pending = false;
  }
  std::vector<void *> allocs;
  Geo geo{};
  Tables<R> tb{};
  R *f[NC] = {}, *fu[NC] = {}, *fw[NC] = {}, *fcnd[NC] = {}, *chi[NC] = {}, *cnd[NC] = {},
    *cndinv[NC] = {};
  // off-diagonal chi1inv of E along d (terms in Plan::offdiag order) and the
  // f_minus_p buffers of the off-diagonal update (one per D component that
  // has polarizations or integrated sources; shared by the two parts of
  // complex fields, which are updated one after the other)
  R *chioff[3][2] = {};
  R *fmp[3] = {};
  struct DPole {
    R *P[3] = {}, *PP[3] = {}, *s[3] = {};
    R *Pim[3] = {}, *PPim[3] = {}; // imaginary parts (complex fields)
    R gamma1inv, gamma1, w0, w0d;
  };
  std::vector<DPole> poles;
  // complex (Bloch) fields: the imaginary parts of every state array; the
  // kernels run once per part with these swapped into f, fu, fw, fcnd, P
  bool cplx = false;
  R *fim[NC] = {}, *fuim[NC] = {}, *fwim[NC] = {}, *fcndim[NC] = {};
  void swap_parts() {
    for (int c = 0; c < NC; c++) {
      std::swap(f[c], fim[c]);
      std::swap(fu[c], fuim[c]);
      std::swap(fw[c], fwim[c]);
      std::swap(fcnd[c], fcndim[c]);
    }
    for (DPole &dp : poles)
      for (int d = 0; d < 3; d++) {
        std::swap(dp.P[d], dp.Pim[d]);
        std::swap(dp.PP[d], dp.PPim[d]);
      }
  }
  // source values for the imaginary part: Re(amp * (-i v)) = Im(amp * v)
  static DipoleVals imag_part(const DipoleVals &v) {
    DipoleVals o = v;
    for (int k = 0; k < 16; k++) {
      o.re[k] = v.im[k];
      o.im[k] = -v.re[k];
    }
    return o;
  }
  // Bloch-periodic ghost plane along d of one array pair, for a component
  // whose shift along d is 0 (shift0) or 1
  void ghost_plane(const Plan &p, int d, bool shift0, R *re, R *im) {
    int o1 = (d + 1) % 3, o2 = (d + 2) % 3;
    if (o1 > o2) std::swap(o1, o2);
    const std::complex<double> ph = shift0 ? std::conj(p.eikna[d]) : p.eikna[d];
    const long long dst = shift0 ? 0 : (long long)p.N[d] * p.stride[d];
    const long long src = shift0 ? (long long)p.N[d] * p.stride[d] : 0;
    const int n1 = p.ext[o1], n2 = p.ext[o2];
    const dim3 grid((unsigned)((n2 + 127) / 128), (unsigned)n1);
    ghost_plane_kernel<R><<<grid, 128, 0, stream>>>(re, im, dst, src, n1, n2, (long long)p.stride[o1],
                                                    (long long)p.stride[o2], R(ph.real()), R(ph.imag()));
    nlaunch++;
  }
  // Bloch-periodic ghost planes of the components of field types t0, t1
  void ghost_copy(const Plan &p, int t0, int t1) {
    for (int d = 0; d < 3; d++) {
      if (!p.periodic[d]) continue;
      for (int c = 0; c < NC; c++) {
        if (!f[c] || (ctype(c) != t0 && ctype(c) != t1)) continue;
        ghost_plane(p, d, p.shift[c][d] == 0, f[c], cplx ? fim[c] : nullptr);
      }
    }
  }
  // polarizations of E at the not-owned points (the reference's PE_stuff
  // boundary step, src/step.cpp:116-119); read by the off-diagonal update
  void ghost_copy_pols(const Plan &p) {
    for (int d = 0; d < 3; d++) {
      if (!p.periodic[d]) continue;
      for (DPole &dp : poles)
        for (int e = 0; e < 3; e++)
          if (dp.P[e]) ghost_plane(p, d, p.shift[comp(MFD_E, e)][d] == 0, dp.P[e], cplx ? dp.Pim[e] : nullptr);
    }
  }
  // sources
  SrcPoint *d_srcpts[3] = {};
  int nsrcpts[3] = {};
  // every integrated E source point of the 3-D step has no active pole and
  // lies outside the E slab of its own direction: its E is set from the
  // final D after the D/E launches (no kernel before them)
  bool src_e_only = false;
  EPoint<R> *d_srcbuf[3] = {};
  DEOut<R> *d_fsrcbuf[3] = {};
  CurPoint *d_cur[NC] = {};
  int ncur[NC] = {};
  // monitors
  struct DMon {
    double2 *acc = nullptr, *ph = nullptr;
    double *freq = nullptr;
    double *w[3] = {};
    bool block = false;      // blocked FP32 contraction
    bool tc = false;         // ... on the tensor cores (3xTF32 tcgen05)
    float *A = nullptr;      // [DFT_BLOCK_T][npts] samples of the current block
    float2 *B = nullptr;     // [DFT_BLOCK_T][nf] phases
    int cnt = 0;             // samples in the current block
    long long tn0 = 0;       // step count of the block's first sample
    // sampled off the main stream: two staging blocks, one filling while
    // the other is contracted; fdone[b] marks the end of block b's contraction
    bool async = false;
    float *Ab[2] = {};
    int cur = 0;
    bool issued[2] = {};
    cudaEvent_t fdone[2] = {};
  };
  std::vector<DMon> mons;
  int *d_tc_err = nullptr; // set by the tensor-core contraction when a wait ran out
  void check_tc() {
    if (!d_tc_err) return;
    int e = 0;
    cuda_check(cudaMemcpyAsync(&e, d_tc_err, sizeof(int), cudaMemcpyDeviceToHost, stream), "error flag");
    cuda_check(cudaStreamSynchronize(stream), "error flag sync");
    if (e) throw Error("tensor-core DFT contraction: an MMA completion wait timed out");
  }
  // divergence test: every finite_every steps (MFD_FINITE_CHECK_EVERY, 0
  // turns it off) the probe kernel checks the centre energy density; the
  // flag is read at the start of every step and after every batch of steps,
  // so a run stops within finite_every steps (plus the steps already queued)
  // of the step the reference would stop at
  int *h_nonfinite = nullptr, *d_nonfinite = nullptr;
  int finite_every = 16;
  void launch_finite_probe(const Plan &p) {
    FiniteProbe<R> fp;
    std::memset(&fp, 0, sizeof(fp));
    for (int d = 0; d < 3; d++) {
      const int ce = comp(MFD_E, d), cd = comp(MFD_D, d);
      if (!f[ce] || !f[cd]) continue;
      const Plan::ProbePoints pp = p.center_probe(d);
      fp.e[d] = f[ce];
      fp.d[d] = f[cd];
      fp.ei[d] = cplx ? fim[ce] : nullptr;
      fp.di[d] = cplx ? fim[cd] : nullptr;
      fp.n[d] = pp.n;
      for (int j = 0; j < pp.n; j++) {
        fp.idx[d][j] = pp.idx[j];
        fp.w[d][j] = pp.w[j];
      }
    }
    fp.flag = d_nonfinite;
    finite_probe_kernel<R><<<1, 1, 0, stream>>>(fp);
    nlaunch++;
    probe_pending = true;
  }
  void check_finite() const {
    if (h_nonfinite && *(volatile int *)h_nonfinite) throw Error("simulation fields are NaN or Inf");
  }
  int fused_mask = -1; // component mask of an available fused kernel set, -1 none
  bool has_b_current = false;
  long long nlaunch = 0;
  double *d_flux = nullptr;
  double *d_flux_part = nullptr;
  size_t flux_cap = 0;
  mutable double ms = 0;
  bool timing = false;

  template <typename T> T *dalloc(size_t n) {
    void *ptr = nullptr;
    if (n == 0) n = 1;
    cuda_check(cudaMalloc(&ptr, n * sizeof(T)), "cudaMalloc");
    allocs.push_back(ptr);
    return (T *)ptr;
  }
  template <typename T> T *dzeros(size_t n) {
    T *ptr = dalloc<T>(n);
    cuda_check(cudaMemsetAsync(ptr, 0, n * sizeof(T), stream), "memset");
    return ptr;
  }
  template <typename T> T *dupload(const std::vector<T> &h) {
    T *ptr = dalloc<T>(h.size());
    cuda_check(cudaMemcpyAsync(ptr, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, stream),
               "upload");
    cuda_check(cudaStreamSynchronize(stream), "sync");
    return ptr;
  }
  std::vector<R> to_store(const Plan &p, const std::vector<double> &dense, double dflt) {
    std::vector<R> out(p.nstore, R(0));
    for (int64_t di = 0; di < p.ndense; di++)
      out[p.store_index_of_dense(di)] = R(dense.empty() ? dflt : dense[di]);
    return out;
  }

  void setup(Plan &p) override {
    p.plan_offdiag();
    if (const char *e = getenv("MFD_FINITE_CHECK_EVERY")) finite_every = std::max(0, atoi(e));
    cuda_check(cudaHostAlloc((void **)&h_nonfinite, sizeof(int), cudaHostAllocMapped), "cudaHostAlloc");
    *(volatile int *)h_nonfinite = 0;
    cuda_check(cudaHostGetDevicePointer((void **)&d_nonfinite, h_nonfinite, 0), "cudaHostGetDevicePointer");
    for (int d = 0; d < 3; d++) {
      geo.N[d] = p.N[d];
      geo.T[d][0] = p.T[d][0];
      geo.T[d][1] = p.T[d][1];
      geo.pml[d] = p.pml_dir[d];
      geo.stride[d] = p.stride[d];
    }
    if (p.g.dim == 3) {
      geo.fast = 2;
      geo.mid = 1;
      geo.slow = 0;
    }
    else if (p.g.dim == 2) {
      geo.fast = 1;
      geo.mid = 0;
      geo.slow = 2;
    }
    else {
      geo.fast = 2;
      geo.mid = 0;
      geo.slow = 1;
    }
    for (int d = 0; d < 3; d++) {
      size_t n = p.sig[d].size();
      std::vector<R> s(n), k(n), si(n);
      for (size_t i = 0; i < n; i++) {
        s[i] = R(p.sig[d][i]);
        k[i] = R(p.kap[d][i]);
        si[i] = (p.sig[d][i] == 0.0 && p.kap[d][i] == 1.0) ? R(1) : R(1) / (k[i] + s[i]);
      }
      tb.sig[d] = dupload(s);
      tb.kap[d] = dupload(k);
      tb.siginv[d] = dupload(si);
    }
    for (int c = 0; c < NC; c++) {
      if (!p.have[c]) continue;
      int t = ctype(c), d = cdir(c);
      f[c] = dzeros<R>(p.nstore);
      if (t == MFD_D || t == MFD_B) {
        const Plan::Curl &cp = p.curl[c];
        if (cp.dsigu >= 0) fu[c] = dzeros<R>(p.nstore);
        if (!p.cond[c].empty()) {
          std::vector<R> cs = to_store(p, p.cond[c], 0.0), ci(p.nstore);
          for (int64_t i = 0; i < p.nstore; i++)
            ci[i] = R(1 / (1 + double(cs[i]) * p.dt * 0.5));
          cnd[c] = dupload(cs);
          cndinv[c] = dupload(ci);
          if (cp.dsig >= 0) fcnd[c] = dzeros<R>(p.nstore);
        }
      }
      if ((t == MFD_E || t == MFD_H) && p.pml_dir[d]) fw[c] = dzeros<R>(p.nstore);
      if (t == MFD_E) {
        chi[c] = dupload(to_store(p, p.chi1inv[c][d], 1.0));
        for (int q = 0; q < p.offdiag[d].n; q++)
          chioff[d][q] = dupload(to_store(p, p.chi1inv[c][p.offdiag[d].dir[q]], 0.0));
      }
      if (t == MFD_H)
        for (int dd = 0; dd < 3; dd++)
          if (!p.chi1inv[c][dd].empty())
            for (double v : p.chi1inv[c][dd])
              if (v != (dd == d ? 1.0 : 0.0)) throw Error("mu != 1 is not supported");
    }
    for (const Pole &pl : p.poles) {
      DPole dp;
      R omega_0 = R(pl.omega0), gamma = R(pl.gamma), dt = R(p.dt);
      const R omega2pi = R(2 * kPi * omega_0), g2pi = R(gamma * 2 * kPi);
      dp.w0 = omega2pi * omega2pi * dt * dt;
      dp.gamma1inv = R(1) / (R(1) + g2pi * dt / R(2));
      dp.gamma1 = (R(1) - g2pi * dt / R(2));
      dp.w0d = pl.drude ? R(0) : dp.w0;
      for (int d = 0; d < 3; d++) {
        int ec = comp(MFD_E, d);
        if (!p.have[ec] || pl.sigma[d].empty()) continue;
        dp.s[d] = dupload(to_store(p, pl.sigma[d], 0.0));
        dp.P[d] = dzeros<R>(p.nstore);
        dp.PP[d] = dzeros<R>(p.nstore);
      }
      poles.push_back(dp);
    }
    cplx = p.complex_fields;
    if (cplx) {
      for (int c = 0; c < NC; c++) {
        if (f[c]) fim[c] = dzeros<R>(p.nstore);
        if (fu[c]) fuim[c] = dzeros<R>(p.nstore);
        if (fw[c]) fwim[c] = dzeros<R>(p.nstore);
        if (fcnd[c]) fcndim[c] = dzeros<R>(p.nstore);
      }
      for (DPole &dp : poles)
        for (int d = 0; d < 3; d++)
          if (dp.P[d]) {
            dp.Pim[d] = dzeros<R>(p.nstore);
            dp.PPim[d] = dzeros<R>(p.nstore);
          }
    }
    setup_sources(p);
    apply_matgrids(p);
    build_active_mask(p);
    if (p.any_offdiag)
      for (int d = 0; d < 3; d++) {
        if (!p.have[comp(MFD_E, d)]) continue;
        bool need = nsrcpts[d] > 0;
        for (const DPole &dp : poles)
          need = need || dp.P[d] != nullptr;
        if (need) fmp[d] = dzeros<R>(p.nstore);
      }
    int mask = 0;
    for (int c = 0; c < NC; c++)
      if (p.have[c]) mask |= 1 << c;
    if ((p.g.dim == 3 && mask == MASK3) || (p.g.dim == 2 && (mask == MASK_TM || mask == MASK_TE)) ||
        (p.g.dim == 1 && mask == MASK_1D))
      fused_mask = mask;
    for (int d = 0; d < 3; d++)
      has_b_current = has_b_current || ncur[comp(MFD_B, d)] > 0;
    if (getenv("MFD_GENERIC_KERNELS")) fused_mask = -1;
    if (p.any_periodic()) fused_mask = -1; // Bloch boundaries: the per-component kernels
    // off-diagonal chi1inv: E needs D - P of all components first; the 3-D
    // band kernels run it as two passes, the 2-D/1-D fused kernels not at all
    if (p.any_offdiag && p.g.dim != 3) fused_mask = -1;
    if (fused_mask >= 0) plan_boxes(p);
    cuda_check(cudaStreamSynchronize(stream), "setup sync");
  }

  // ---------------------------------------------------- material grids
  MGPoints mg_points(const Plan &p, int c, const int lo[3], const int hi[3]) const {
    MGPoints a;
    for (int d = 0; d < 3; d++) {
      a.lo[d] = lo[d];
      a.n[d] = hi[d] - lo[d] + 1;
      a.io[d] = p.g.io[d];
      a.sh[d] = p.shift[c][d];
      a.present[d] = p.present[d];
      a.stride[d] = p.stride[d];
    }
    a.inva = p.inva;
    return a;
  }
  // the projected weights of every material grid into the diagonal chi1inv
  // of the E components, grids in order
  void apply_matgrids(const Plan &p) {
    for (int id = 0; id < int(p.matgrids.size()); id++) {
      const Plan::MatGrid &mg = p.matgrids[id];
      double *du = dupload(mg.u);
      for (int d = 0; d < 3; d++) {
        const int c = comp(MFD_E, d);
        if (!p.have[c]) continue;
        int lo[3], hi[3];
        p.matgrid_box(id, c, lo, hi);
        if (lo[0] > hi[0] || lo[1] > hi[1] || lo[2] > hi[2]) continue; // block outside the cell
        const MGPoints a = mg_points(p, c, lo, hi);
        const long long n = (long long)a.n[0] * a.n[1] * a.n[2];
        matgrid_chi_kernel<R><<<unsigned((n + 255) / 256), 256, 0, stream>>>(a, mg.spec, du, d, chi[c]);
        cuda_check(cudaGetLastError(), "matgrid_chi_kernel");
        nlaunch++;
      }
    }
    cuda_check(cudaStreamSynchronize(stream), "material grids");
  }
  void matgrid_vjp(Plan &p, int id, const std::vector<int> &comps, const int lo[3], const int hi[3],
                   const double *gchi, double *gu) override {
    join_dft();
    const Plan::MatGrid &mg = p.matgrids[id];
    std::vector<MatGridSpec> specs;
    for (const Plan::MatGrid &m : p.matgrids)
      specs.push_back(m.spec);
    const long long nbox = (long long)(hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1);
    const long long nu = (long long)mg.spec.n[0] * mg.spec.n[1] * mg.spec.n[2];
    std::vector<void *> tmp;
    auto alloc = [&](size_t bytes) {
      void *ptr = nullptr;
      cuda_check(cudaMalloc(&ptr, bytes ? bytes : 1), "cudaMalloc");
      tmp.push_back(ptr);
      return ptr;
    };
    try {
      MatGridSpec *dspec = (MatGridSpec *)alloc(specs.size() * sizeof(MatGridSpec));
      double *du = (double *)alloc(nu * sizeof(double));
      double *dg = (double *)alloc(comps.size() * nbox * sizeof(double));
      double *drho = (double *)alloc(nbox * sizeof(double));
      double *dgu = (double *)alloc(nu * sizeof(double));
      cuda_check(cudaMemcpyAsync(dspec, specs.data(), specs.size() * sizeof(MatGridSpec), cudaMemcpyHostToDevice,
                                 stream), "upload");
      cuda_check(cudaMemcpyAsync(du, mg.u.data(), nu * sizeof(double), cudaMemcpyHostToDevice, stream), "upload");
      cuda_check(cudaMemcpyAsync(dg, gchi, comps.size() * nbox * sizeof(double), cudaMemcpyHostToDevice, stream),
                 "upload");
      for (size_t q = 0; q < comps.size(); q++) {
        const int c = comps[q];
        const MGPoints a = mg_points(p, c, lo, hi);
        matgrid_grho_kernel<<<unsigned((nbox + 255) / 256), 256, 0, stream>>>(
            a, dspec, int(specs.size()), id, du, c % 3, dg + q * nbox, drho);
        cuda_check(cudaGetLastError(), "matgrid_grho_kernel");
        matgrid_gather_kernel<<<unsigned((nu + 127) / 128), 128, 0, stream>>>(a, mg.spec, drho, dgu, q > 0);
        cuda_check(cudaGetLastError(), "matgrid_gather_kernel");
        nlaunch += 2;
      }
      cuda_check(cudaMemcpyAsync(gu, dgu, nu * sizeof(double), cudaMemcpyDeviceToHost, stream), "download");
      cuda_check(cudaStreamSynchronize(stream), "material grid gradient");
    } catch (...) {
      for (void *ptr : tmp)
        cudaFree(ptr);
      throw;
    }
    for (void *ptr : tmp)
      cudaFree(ptr);
  }

  // activity bits per row segment of 32 z points (FusedArgs::amask) for
  // the 3-D band kernels: poles with a nonzero sigma and D/B components with
  // a nonzero conductivity somewhere in the segment
  unsigned *d_amask = nullptr;
  int amask_nseg = 0;
  std::vector<unsigned> h_amask;
  // the activity word shared by every segment that holds points of the
  // bands, with bit 31 set; 0 when they differ
  unsigned uniform_am(std::initializer_list<Band> bands) const {
    if (h_amask.empty()) return 0u;
    const int nseg = amask_nseg, ext1 = (int)(h_amask.size() / nseg) / std::max(1, geo_ext0);
    // the two runs [lo, hi) of a span
    auto runs = [](const Span &z, int r[2][2]) {
      r[0][0] = z.a0, r[0][1] = z.a0 + z.split;
      r[1][0] = z.a1 + z.split, r[1][1] = z.a1 + z.n;
    };
    bool first = true;
    unsigned w = 0;
    for (const Band &b : bands) {
      if (b.s[0].n <= 0 || b.s[1].n <= 0 || b.s[2].n <= 0) continue;
      int rx[2][2], ry[2][2], rz[2][2];
      runs(b.s[0], rx);
      runs(b.s[1], ry);
      runs(b.s[2], rz);
      for (const auto &x : rx)
        for (int k0 = x[0]; k0 < x[1]; k0++)
          for (const auto &y : ry)
            for (int k1 = y[0]; k1 < y[1]; k1++)
              for (const auto &z : rz) {
                if (z[1] <= z[0]) continue;
                for (int g = z[0] / 32; g <= (z[1] - 1) / 32; g++) {
                  const unsigned v = h_amask[((size_t)k0 * ext1 + k1) * nseg + g];
                  if (first) w = v, first = false;
                  else if (v != w) return 0u;
                }
              }
    }
    return first ? 0u : (w | (1u << 31));
  }
  int geo_ext0 = 1;
  void build_active_mask(const Plan &p) {
    if (p.g.dim != 3) return;
    bool any = !poles.empty();
    for (int d = 0; d < 3; d++)
      any = any || cnd[comp(MFD_D, d)] || cnd[comp(MFD_B, d)];
    if (!any) return;
    geo_ext0 = p.ext[0];
    const int nseg = (p.ext[2] + 31) / 32;
    std::vector<unsigned> m((size_t)p.ext[0] * p.ext[1] * nseg, 0u);
    auto mark = [&](const std::vector<double> &dense, unsigned bit) {
      if (dense.empty()) return;
      int64_t di = 0;
      for (int k0 = 0; k0 < p.ext[0]; k0++)
        for (int k1 = 0; k1 < p.ext[1]; k1++) {
          unsigned *row = &m[((size_t)k0 * p.ext[1] + k1) * nseg];
          for (int k2 = 0; k2 < p.ext[2]; k2++, di++)
            if (dense[di] != 0.0) row[k2 >> 5] |= bit;
        }
    };
    for (size_t q = 0; q < poles.size(); q++)
      for (int d = 0; d < 3; d++)
        if (poles[q].P[d]) mark(p.poles[q].sigma[d], 1u << (3 * q + d));
    for (int d = 0; d < 3; d++) {
      if (cnd[comp(MFD_D, d)]) mark(p.cond[comp(MFD_D, d)], 1u << (12 + d));
      if (cnd[comp(MFD_B, d)]) mark(p.cond[comp(MFD_B, d)], 1u << (15 + d));
    }
    d_amask = dupload(m);
    amask_nseg = nseg;
    h_amask = m;
    // z extent of the segments where some pole is active anywhere: rows
    // outside it take the pole-free D/E kernel
    const unsigned pole_bits = (1u << (3 * MAX_POLES)) - 1u;
    int s0 = nseg, s1 = -1;
    for (size_t c = 0; c < m.size(); c++)
      if (m[c] & pole_bits) {
        const int sg = (int)(c % nseg);
        s0 = std::min(s0, sg);
        s1 = std::max(s1, sg);
      }
    pole_z0 = s1 >= s0 ? 32 * s0 : 0;
    pole_z1 = s1 >= s0 ? std::min(32 * (s1 + 1), p.ext[2]) : 0;
  }
  int pole_z0 = 0, pole_z1 = -1; // z points [pole_z0, pole_z1) hold every active pole (-1: unknown)
  // uniform activity words of the pole rows, the pole-free rows and the
  // pole-free z interior of the faces (0: loaded per segment)
  unsigned bp_am = 0, bn_am = 0, qf_am = 0;
  bool bp_am_done = false, bn_am_done = false, qf_am_done = false;

  static constexpr int MASK3 = 0xFFF;
  static constexpr int MASK_TM = (1 << 2) | (1 << 3) | (1 << 4) | (1 << 8) | (1 << 9) | (1 << 10);
  static constexpr int MASK_TE = (1 << 0) | (1 << 1) | (1 << 5) | (1 << 6) | (1 << 7) | (1 << 11);
  static constexpr int MASK_1D = (1 << 0) | (1 << 4) | (1 << 6) | (1 << 10);

  FusedArgs<R> fused_args(const Plan &p, bool fuse_h) {
    FusedArgs<R> a;
    std::memset(&a, 0, sizeof(a));
    for (int d = 0; d < 3; d++) {
      a.e[d] = f[comp(MFD_E, d)];
      a.d[d] = f[comp(MFD_D, d)];
      a.b[d] = f[comp(MFD_B, d)];
      a.h[d] = f[comp(MFD_H, d)];
      for (int t = 2; t < 4; t++) {
        int c = comp(t, d);
        a.fu[t][d] = fu[c];
        a.fcnd[t][d] = fcnd[c];
        a.cnd[t][d] = cnd[c];
        a.cndinv[t][d] = cndinv[c];
        unsigned m = 0;
        if (!p.cond_chunk[c].empty())
          for (int r = 0; r < 27; r++)
            if (p.cond_chunk[c][r]) m |= 1u << r;
        a.cond_chunks[t][d] = m;
      }
      a.fw[0][d] = fw[comp(MFD_E, d)];
      a.fw[1][d] = fw[comp(MFD_H, d)];
      a.chi[d] = chi[comp(MFD_E, d)];
      a.N[d] = p.N[d];
      a.T[d][0] = p.T[d][0];
      a.T[d][1] = p.T[d][1];
      a.pml[d] = p.pml_dir[d];
      a.s[d] = (int)p.stride[d];
      a.sig[d] = tb.sig[d];
      a.kap[d] = tb.kap[d];
      a.siginv[d] = tb.siginv[d];
    }
    a.npoles = (int)poles.size();
    for (int q = 0; q < a.npoles; q++) {
      for (int d = 0; d < 3; d++) {
        a.P[q][d] = poles[q].P[d];
        a.PP[q][d] = poles[q].PP[d];
        a.ps[q][d] = poles[q].s[d];
      }
      a.pg1inv[q] = poles[q].gamma1inv;
      a.pg1[q] = poles[q].gamma1;
      a.pw0[q] = poles[q].w0;
      a.pw0d[q] = poles[q].w0d;
    }
    a.dtdx = R(p.g.courant);
    a.dt2 = R(p.dt) * R(0.5);
    a.fuse_h = fuse_h;
    a.amask = d_amask;
    a.mext1 = p.ext[1];
    a.mnseg = amask_nseg;
    for (int d = 0; d < 3; d++) {
      a.fmp[d] = fmp[d];
      a.noff[d] = p.offdiag[d].n;
      for (int q = 0; q < p.offdiag[d].n; q++) {
        a.chio[d][q] = chioff[d][q];
        a.odir[d][q] = p.offdiag[d].dir[q];
        a.osx[d][q] = (int)p.stride[p.offdiag[d].dir[q]];
      }
    }
    return a;
  }

  // Interior box (no PML slab, no wall point for any component) and the boxes
  // around it, in point indices 0..N-1 per present direction.
  BoxList box_int{}, box_bnd{};
  dim3 fblock{32, 8, 1};

  // 3-D decomposition: rows (x, y interior, all z; z slabs inside the rows),
  // x slabs (all y, all z), y slabs (interior x, all z).  The FP32 B update
  // splits the rows into the core (quads) and the z ends of the rows.
  // slabs split by how many directions can hold slab points: faces (one) run
  // the lean single-flag code, edges and corners the general code
  Band band_rows{}, band_zend{}, band_xface{}, band_yface{}, band_xyedge{};
  // FP64 (issue-bound) shell: faces over the z interior only (no z flags) and
  // the z edges of the faces
  Band band_xface_zi{}, band_yface_zi{}, band_xzedge{}, band_yzedge{};
  // FP32: the z-interior faces of the B half-step as quads (QFaces) when
  // their z run is whole quads; the B shell launch then leaves them out
  QFaces qfaces{};
  bool use_qfaces = false;

  // the rows without their z slabs and walls (z range of the quad core): no
  // PML flag in any direction; band_zend holds the rest of the rows
  Band band_core{};
  QCore qcore{};

  static Span span_run(int lo, int hi) {
    Span s{};
    s.n = std::max(0, hi - lo + 1);
    s.split = s.n;
    s.a0 = lo;
    return s;
  }
  // points 0..n-1 outside the run lo..hi
  static Span span_outside(int n, int lo, int hi) {
    Span s{};
    s.split = lo;
    s.n = lo + (n - 1 - hi);
    s.a0 = 0;
    s.a1 = hi + 1 - lo;
    return s;
  }
  // the points of s in [z0, z1)
  static Span span_clip(const Span &s, int z0, int z1) {
    const int lo0 = std::max(s.a0, z0), hi0 = std::min(s.a0 + s.split, z1);
    const int lo1 = std::max(s.a1 + s.split, z0), hi1 = std::min(s.a1 + s.n, z1);
    const int n0 = std::max(0, hi0 - lo0), n1 = std::max(0, hi1 - lo1);
    if (n0 > 0 && n1 > 0) {
      Span r{};
      r.n = n0 + n1;
      r.split = n0;
      r.a0 = lo0;
      r.a1 = lo1 - n0;
      return r;
    }
    if (n0 > 0) return span_run(lo0, hi0 - 1);
    if (n1 > 0) return span_run(lo1, hi1 - 1);
    return span_run(0, -1);
  }
  // short z spans (the z ends of the rows) take whole blocks of several rows
  // so no lane idles; long spans take warps of 32 consecutive z points
  static void band_shape(const Band &b, dim3 &g, dim3 &blk) {
    g = blk = dim3(0, 0, 0);
    if (b.s[0].n <= 0 || b.s[1].n <= 0 || b.s[2].n <= 0) return;
    if (b.s[2].n <= 64) {
      blk = dim3((unsigned)b.s[2].n, (unsigned)std::max(1, 256 / b.s[2].n), 1);
      g = dim3(1, (unsigned)((b.s[1].n + blk.y - 1) / blk.y), (unsigned)b.s[0].n);
      return;
    }
    blk = dim3(32, 8, 1);
    g = dim3((unsigned)((b.s[2].n + 31) / 32), (unsigned)((b.s[1].n + 7) / 8), (unsigned)b.s[0].n);
  }

  // ZCAN: the band can hold z slab points (the z flags are computed when the
  // grid has a z PML)
  template <bool FX, bool FY, bool ZCAN = true>
  void launch_b_band(const Band &bd, const FusedArgs<R> &a, bool cnd, bool zp_, cudaStream_t st) {
    const bool zp = ZCAN && zp_;
    dim3 g, blk;
    band_shape(bd, g, blk);
    if (g.x == 0) return;
    if (cnd && zp) b3_band_kernel<R, true, FX, FY, true><<<g, blk, 0, st>>>(a, bd);
    else if (cnd) b3_band_kernel<R, true, FX, FY, false><<<g, blk, 0, st>>>(a, bd);
    else if (zp) b3_band_kernel<R, false, FX, FY, true><<<g, blk, 0, st>>>(a, bd);
    else b3_band_kernel<R, false, FX, FY, false><<<g, blk, 0, st>>>(a, bd);
    nlaunch++;
  }
  template <bool FX, bool FY, int NP>
  void launch_de_band_p(const Band &bd, const dim3 &g, const dim3 &blk, const FusedArgs<R> &a, bool cnd, bool zp,
                        cudaStream_t st) {
    if (cnd && zp) de3_band_kernel<R, true, NP, FX, FY, true><<<g, blk, 0, st>>>(a, bd);
    else if (cnd) de3_band_kernel<R, true, NP, FX, FY, false><<<g, blk, 0, st>>>(a, bd);
    else if (zp) de3_band_kernel<R, false, NP, FX, FY, true><<<g, blk, 0, st>>>(a, bd);
    else de3_band_kernel<R, false, NP, FX, FY, false><<<g, blk, 0, st>>>(a, bd);
  }
  // ZCAN: the band can hold z slab points (the z flags are computed when the
  // grid has a z PML)
  template <bool FX, bool FY, bool ZCAN = true>
  void launch_de_band(const Band &bd, const FusedArgs<R> &a, bool cnd, bool zp_, cudaStream_t st) {
    const bool zp = ZCAN && zp_;
    dim3 g, blk;
    band_shape(bd, g, blk);
    if (g.x == 0) return;
    // up to two poles in registers, more one component after the other
    if (a.npoles == 1) launch_de_band_p<FX, FY, 1>(bd, g, blk, a, cnd, zp, st);
    else if (a.npoles == 2) launch_de_band_p<FX, FY, 2>(bd, g, blk, a, cnd, zp, st);
    else if (a.npoles > 2) launch_de_band_p<FX, FY, -1>(bd, g, blk, a, cnd, zp, st);
    else launch_de_band_p<FX, FY, 0>(bd, g, blk, a, cnd, zp, st);
    nlaunch++;
  }

  // the shell bands of a half-step as one launch (ShellSet)
  // skip_zi: the z-interior faces run elsewhere (FP32: quads); zi: their z
  // span when only part of it stays in the shell (null: all of it)
  // z0, z1: only the points with z in [z0, z1)
  ShellSet shell_set(bool skip_zi, const Span *zi = nullptr, int z0 = 0, int z1 = 1 << 30) const {
    ShellSet s{};
    const Band *bands[5] = {&band_xface_zi, &band_yface_zi, &band_xzedge, &band_yzedge, &band_xyedge};
    int total = 0;
    for (int q = 0; q < 5; q++) {
      Band b = *bands[q];
      if (zi && q < 2) b.s[2] = *zi;
      if (z0 > 0 || z1 < (1 << 30)) b.s[2] = span_clip(b.s[2], z0, z1);
      s.b[q] = b;
      const bool empty = b.s[0].n <= 0 || b.s[1].n <= 0 || b.s[2].n <= 0 || (skip_zi && q < 2);
      s.gz[q] = empty ? 1 : (b.s[2].n + 31) / 32;
      s.gy[q] = empty ? 1 : (b.s[1].n + 7) / 8;
      s.first[q] = total;
      if (!empty) total += s.gz[q] * s.gy[q] * b.s[0].n;
    }
    s.first[5] = total;
    return s;
  }
  void launch_b_shell(const FusedArgs<R> &a, bool cnd, bool zp, cudaStream_t st) {
    const ShellSet s = shell_set(use_qfaces);
    if (s.first[5] == 0) return;
    const dim3 g(s.first[5]), blk(32, 8);
    if (cnd && zp) b3_shell_kernel<R, true, true><<<g, blk, 0, st>>>(a, s);
    else if (cnd) b3_shell_kernel<R, true, false><<<g, blk, 0, st>>>(a, s);
    else if (zp) b3_shell_kernel<R, false, true><<<g, blk, 0, st>>>(a, s);
    else b3_shell_kernel<R, false, false><<<g, blk, 0, st>>>(a, s);
    nlaunch++;
  }
  template <int NP> void launch_de_shell_p(const ShellSet &s, const FusedArgs<R> &a, bool cnd, bool zp,
                                           cudaStream_t st) {
    const dim3 g(s.first[5]), blk(32, 8);
    if (cnd && zp) de3_shell_kernel<R, true, NP, true><<<g, blk, 0, st>>>(a, s);
    else if (cnd) de3_shell_kernel<R, true, NP, false><<<g, blk, 0, st>>>(a, s);
    else if (zp) de3_shell_kernel<R, false, NP, true><<<g, blk, 0, st>>>(a, s);
    else de3_shell_kernel<R, false, NP, false><<<g, blk, 0, st>>>(a, s);
  }
  // the D/E shell with the poles in z [pole_z0, pole_z1) cut at pole_z1
  // (pole_z0 = 0): the part below with the pole kernel, the part above with
  // the pole-free one, each with its segments' activity word when uniform
  ShellSet sh_lo{}, sh_hi{};
  unsigned sh_lo_am = 0, sh_hi_am = 0;
  bool sh_done = false;
  void launch_de_shell_split(const FusedArgs<R> &a, bool cnd, bool zp, const Span *zi) {
    if (pole_z0 != 0 || a.npoles > 2) {
      launch_de_shell(a, cnd, zp, false, S(0), zi);
      return;
    }
    if (!sh_done) {
      sh_lo = shell_set(false, zi, 0, pole_z1);
      sh_hi = shell_set(false, zi, pole_z1, 1 << 30);
      auto am_of = [&](const ShellSet &ss) {
        return uniform_am({ss.b[0], ss.b[1], ss.b[2], ss.b[3], ss.b[4]});
      };
      sh_lo_am = am_of(sh_lo);
      sh_hi_am = am_of(sh_hi);
      sh_done = true;
    }
    FusedArgs<R> al = a, ah = a;
    al.am_all = sh_lo_am;
    ah.am_all = sh_hi_am;
    if (sh_lo.first[5] > 0) {
      if (a.npoles == 1) launch_de_shell_p<1>(sh_lo, al, cnd, zp, S(0));
      else launch_de_shell_p<2>(sh_lo, al, cnd, zp, S(0));
      nlaunch++;
    }
    if (sh_hi.first[5] > 0) {
      launch_de_shell_p<0>(sh_hi, ah, cnd, zp, S(3));
      nlaunch++;
    }
  }
  void launch_de_shell(const FusedArgs<R> &a, bool cnd, bool zp, bool skip_zi, cudaStream_t st,
                       const Span *zi = nullptr) {
    const ShellSet s = shell_set(skip_zi, zi);
    if (s.first[5] == 0) return;
    if (a.npoles == 1) launch_de_shell_p<1>(s, a, cnd, zp, st);
    else if (a.npoles == 2) launch_de_shell_p<2>(s, a, cnd, zp, st);
    else if (a.npoles > 2) launch_de_shell_p<-1>(s, a, cnd, zp, st);
    else launch_de_shell_p<0>(s, a, cnd, zp, st);
    nlaunch++;
  }

  // FP32 D/E faces as quads where no pole is active (over the z run zq of
  // the z interior, or all of it; the shell takes the rest); true if launched
  bool launch_de_qfaces(const FusedArgs<R> &a, bool cnd, cudaStream_t st, const Span *zq = nullptr) {
    if constexpr (std::is_same<R, float>::value) {
      if (!use_qfaces || (a.npoles != 0 && !zq)) return false;
      QFaces f = qfaces;
      if (zq) {
        for (int q = 0; q < 2; q++) {
          f.b[q].s[2] = *zq;
          f.nq[q] = zq->n / 4;
          f.nquads[q] = f.b[q].s[0].n > 0 && f.b[q].s[1].n > 0 ? (long long)f.b[q].s[0].n * f.b[q].s[1].n * f.nq[q]
                                                              : 0;
          f.nblk[q] = (int)((f.nquads[q] + 255) / 256);
        }
        if (f.nblk[0] + f.nblk[1] == 0) return false;
      }
      const dim3 g(f.nblk[0] + f.nblk[1]);
      if (cnd) de3q_faces_kernel<true><<<g, 256, 0, st>>>(a, f);
      else de3q_faces_kernel<false><<<g, 256, 0, st>>>(a, f);
      nlaunch++;
      return true;
    }
    return false;
  }
  // FP64 (issue-bound): the shell bands as separate launches on the side
  // streams (one launch per half-step ran 2.5% slower there)
  void launch_b_shell_bands(const FusedArgs<R> &a, bool cnd, bool zp) {
    launch_b_band<true, false, false>(band_xface_zi, a, cnd, zp, S(0));
    launch_b_band<false, true, false>(band_yface_zi, a, cnd, zp, S(1));
    launch_b_band<true, false>(band_xzedge, a, cnd, zp, S(4));
    launch_b_band<false, true>(band_yzedge, a, cnd, zp, S(5));
    launch_b_band<true, true>(band_xyedge, a, cnd, zp, S(3));
  }
  void launch_de_shell_bands(const FusedArgs<R> &a, bool cnd, bool zp) {
    launch_de_band<true, false, false>(band_xface_zi, a, cnd, zp, S(0));
    launch_de_band<false, true, false>(band_yface_zi, a, cnd, zp, S(1));
    launch_de_band<true, false>(band_xzedge, a, cnd, zp, S(4));
    launch_de_band<false, true>(band_yzedge, a, cnd, zp, S(5));
    launch_de_band<true, true>(band_xyedge, a, cnd, zp, S(3));
  }
  void launch_b_qfaces(const FusedArgs<R> &a, bool cnd, cudaStream_t st) {
    if constexpr (std::is_same<R, float>::value) {
      if (!use_qfaces) return;
      const dim3 g(qfaces.nblk[0] + qfaces.nblk[1]);
      if (cnd) b3q_faces_kernel<true><<<g, 256, 0, st>>>(a, qfaces);
      else b3q_faces_kernel<false><<<g, 256, 0, st>>>(a, qfaces);
      nlaunch++;
    }
  }
  // the two passes of the off-diagonal D/E half-step (3-D)
  template <bool FX, bool FY, bool ZCAN = true>
  void launch_d_band(const Band &bd, const FusedArgs<R> &a, bool cnd, bool zp_, cudaStream_t st) {
    const bool zp = ZCAN && zp_;
    dim3 g, blk;
    band_shape(bd, g, blk);
    if (g.x == 0) return;
    if (cnd && zp) d3_band_kernel<R, true, FX, FY, true><<<g, blk, 0, st>>>(a, bd);
    else if (cnd) d3_band_kernel<R, true, FX, FY, false><<<g, blk, 0, st>>>(a, bd);
    else if (zp) d3_band_kernel<R, false, FX, FY, true><<<g, blk, 0, st>>>(a, bd);
    else d3_band_kernel<R, false, FX, FY, false><<<g, blk, 0, st>>>(a, bd);
    nlaunch++;
  }
  template <bool FX, bool FY, bool ZCAN = true>
  void launch_e_band(const Band &bd, const FusedArgs<R> &a, bool zp_, cudaStream_t st) {
    const bool zp = ZCAN && zp_;
    dim3 g, blk;
    band_shape(bd, g, blk);
    if (g.x == 0) return;
    const bool poles = a.npoles > 0;
    if (poles && zp) e3_band_kernel<R, true, FX, FY, true><<<g, blk, 0, st>>>(a, bd);
    else if (poles) e3_band_kernel<R, true, FX, FY, false><<<g, blk, 0, st>>>(a, bd);
    else if (zp) e3_band_kernel<R, false, FX, FY, true><<<g, blk, 0, st>>>(a, bd);
    else e3_band_kernel<R, false, FX, FY, false><<<g, blk, 0, st>>>(a, bd);
    nlaunch++;
  }
  // launches one pass over rows + shell (the shell on the side streams)
  template <class F> void over_bands3(const Plan &p, F &&launch) {
    (void)p;
    fork();
    launch(band_rows, 0, stream);
    launch(band_xface_zi, 4, S(0));
    launch(band_yface_zi, 5, S(1));
    launch(band_xzedge, 6, S(4));
    launch(band_yzedge, 7, S(5));
    launch(band_xyedge, 3, S(3));
    join();
  }
  void offdiag_de3(const Plan &p, const FusedArgs<R> &a, bool cnd, bool zp, const DipoleVals &dip) {
    // kind: 0 rows, 1 full-row x faces, 2 full-row y faces, 3 xy edges,
    // 4/5 z-interior x/y faces, 6/7 their z edges
    over_bands3(p, [&](const Band &b, int kind, cudaStream_t st) {
      switch (kind) {
        case 0: launch_d_band<false, false>(b, a, cnd, zp, st); break;
        case 1: launch_d_band<true, false>(b, a, cnd, zp, st); break;
        case 2: launch_d_band<false, true>(b, a, cnd, zp, st); break;
        case 3: launch_d_band<true, true>(b, a, cnd, zp, st); break;
        case 4: launch_d_band<true, false, false>(b, a, cnd, zp, st); break;
        case 5: launch_d_band<false, true, false>(b, a, cnd, zp, st); break;
        case 6: launch_d_band<true, false>(b, a, cnd, zp, st); break;
        default: launch_d_band<false, true>(b, a, cnd, zp, st); break;
      }
    });
    for (int d = 0; d < 3; d++)
      if (nsrcpts[d] && fmp[d]) {
        FmpArgs<R> fa{};
        fa.out = fmp[d];
        fa.d = f[comp(MFD_D, d)];
        fa.np = (int)poles.size();
        for (int q = 0; q < fa.np; q++)
          fa.p[q] = poles[q].P[d];
        src_fmp_kernel<R><<<(nsrcpts[d] + 127) / 128, 128, 0, stream>>>(fa, d_srcpts[d], nsrcpts[d], dip);
        nlaunch++;
      }
    over_bands3(p, [&](const Band &b, int kind, cudaStream_t st) {
      switch (kind) {
        case 0: launch_e_band<false, false>(b, a, zp, st); break;
        case 1: launch_e_band<true, false>(b, a, zp, st); break;
        case 2: launch_e_band<false, true>(b, a, zp, st); break;
        case 3: launch_e_band<true, true>(b, a, zp, st); break;
        case 4: launch_e_band<true, false, false>(b, a, zp, st); break;
        case 5: launch_e_band<false, true, false>(b, a, zp, st); break;
        case 6: launch_e_band<true, false>(b, a, zp, st); break;
        default: launch_e_band<false, true>(b, a, zp, st); break;
      }
    });
  }

  dim3 core_grid() const {
    if (qcore.total <= 0) return dim3(0, 0, 0);
    return dim3((unsigned)((qcore.total + 255) / 256), 1, 1);
  }

  static void add_box(BoxList &L, const int lo[3], const int hi[3], int dim, dim3 blk) {
    int ext[3];
    for (int d = 0; d < 3; d++) {
      ext[d] = hi[d] - lo[d] + 1;
      if (ext[d] <= 0) return;
    }
    const int FA = dim == 2 ? 1 : 2, MA = dim == 2 ? 0 : (dim == 3 ? 1 : 0), SA = dim == 3 ? 0 : (dim == 2 ? 2 : 1);
    if (L.n >= 7) throw Error("internal: too many boxes");
    int q = L.n++;
    for (int d = 0; d < 3; d++) {
      L.lo[q][d] = lo[d];
      L.ext[q][d] = ext[d];
    }
    L.bx[q] = (ext[FA] + blk.x - 1) / blk.x;
    L.by[q] = (ext[MA] + blk.y - 1) / blk.y;
    L.blk0[q + 1] = L.blk0[q] + L.bx[q] * L.by[q] * ext[SA];
  }

  void plan_boxes(const Plan &p) {
    if (p.nstore >= (1LL << 31)) throw Error("grid too large for 32-bit indexing");
    const int dim = p.g.dim;
    fblock = dim == 1 ? dim3(256, 1, 1) : dim3(32, 8, 1);
    int glo[3], ghi[3], ilo[3], ihi[3];
    for (int d = 0; d < 3; d++) {
      if (!p.present[d]) {
        glo[d] = ghi[d] = ilo[d] = ihi[d] = 0;
        continue;
      }
      glo[d] = 0;
      ghi[d] = p.N[d] - 1;
      ilo[d] = p.T[d][0] + 1;
      ihi[d] = p.N[d] - p.T[d][1] - 1;
      if (d == p.fastdir && dim > 1) {
        // whole warps along the unit-stride axis: interior rows start and end
        // on multiples of 32 points (the shell takes the remainder)
        ilo[d] = (ilo[d] + 31) / 32 * 32;
        ihi[d] = (ihi[d] + 1) / 32 * 32 - 1;
      }
      if (ilo[d] > ghi[d] + 1) ilo[d] = ghi[d] + 1;
      if (ihi[d] < ilo[d]) ihi[d] = ilo[d] - 1; // empty interior
    }
    box_int = BoxList{};
    box_bnd = BoxList{};
    if (dim == 3) {
      int xlo = p.T[0][0] + 1, xhi = p.N[0] - p.T[0][1] - 1, ylo = p.T[1][0] + 1, yhi = p.N[1] - p.T[1][1] - 1;
      xlo = std::min(xlo, p.N[0]);
      ylo = std::min(ylo, p.N[1]);
      xhi = std::max(xhi, xlo - 1);
      yhi = std::max(yhi, ylo - 1);
      band_rows = Band{{span_run(xlo, xhi), span_run(ylo, yhi), span_run(0, p.N[2] - 1)}};
      const Span sxr = span_run(xlo, xhi), sxo = span_outside(p.N[0], xlo, xhi);
      const Span syr = span_run(ylo, yhi), syo = span_outside(p.N[1], ylo, yhi);
      const Span sza = span_run(0, p.N[2] - 1);
      // the x and y slabs take whole z rows (warps start on 128-byte
      // boundaries; the z slabs ride along on the z flags)
      band_xface = Band{{sxo, syr, sza}};
      band_yface = Band{{sxr, syo, sza}};
      band_xyedge = Band{{sxo, syo, sza}};
      int zlo = std::min(p.T[2][0] + 1, p.N[2]), zhi = p.N[2] - p.T[2][1] - 1;
      zhi = std::max(zhi, zlo - 1);
      if (std::is_same<R, float>::value) {
        // FP32: the z interior rounded inwards to whole warps of 32 points
        // (every warp of the face bands starts on a 128-byte line)
        const int zl = (zlo + 31) / 32 * 32, zh = (zhi + 1) / 32 * 32 - 1;
        if (zh >= zl) {
          zlo = zl;
          zhi = zh;
        }
      }
      const Span szr = span_run(zlo, zhi), szo = span_outside(p.N[2], zlo, zhi);
      band_xface_zi = Band{{sxo, syr, szr}};
      band_yface_zi = Band{{sxr, syo, szr}};
      band_xzedge = Band{{sxo, syr, szo}};
      band_yzedge = Band{{sxr, syo, szo}};
      use_qfaces = false;
      if (std::is_same<R, float>::value && szr.n > 0 && szr.a0 % 4 == 0 && szr.n % 4 == 0 && p.stride[2] == 1 &&
          p.stride[1] % 4 == 0 && p.stride[0] % 4 == 0) {
        qfaces = QFaces{};
        const Band *fb[2] = {&band_xface_zi, &band_yface_zi};
        for (int f = 0; f < 2; f++) {
          qfaces.b[f] = *fb[f];
          qfaces.nq[f] = szr.n / 4;
          qfaces.nquads[f] = fb[f]->s[0].n > 0 && fb[f]->s[1].n > 0
                                 ? (long long)fb[f]->s[0].n * fb[f]->s[1].n * qfaces.nq[f]
                                 : 0;
          qfaces.nblk[f] = (int)((qfaces.nquads[f] + 255) / 256);
        }
        use_qfaces = qfaces.nblk[0] + qfaces.nblk[1] > 0;
      }
      // the B core: z interior (no slab, off the low wall) rounded inwards to quads
      qcore = QCore{};
      qcore.lo[0] = xlo;
      qcore.lo[1] = ylo;
      qcore.n[0] = xhi - xlo + 1;
      qcore.n[1] = yhi - ylo + 1;
      qcore.lo[2] = (std::max(p.T[2][0] + 1, 1) + 3) / 4 * 4;
      qcore.zend = std::max((p.N[2] - p.T[2][1]) / 4 * 4, qcore.lo[2]);
      qcore.nq = (qcore.zend - qcore.lo[2]) / 4;
      qcore.total = qcore.nq > 0 && qcore.n[0] > 0 && qcore.n[1] > 0
                        ? (long long)qcore.n[0] * qcore.n[1] * qcore.nq
                        : 0;
      band_zend = Band{{span_run(xlo, xhi), span_run(ylo, yhi),
                        qcore.zend > qcore.lo[2] ? span_outside(p.N[2], qcore.lo[2], qcore.zend - 1)
                                                 : span_run(0, p.N[2] - 1)}};
      band_core = qcore.zend > qcore.lo[2]
                      ? Band{{span_run(xlo, xhi), span_run(ylo, yhi), span_run(qcore.lo[2], qcore.zend - 1)}}
                      : Band{{span_run(0, -1), span_run(0, -1), span_run(0, -1)}};
      check_bands(p);
      return;
    }
    add_box(box_int, ilo, ihi, dim, fblock);
    // shell around the interior: slabs peeled off direction by direction
    int lo[3], hi[3], clo[3], chi_[3];
    for (int d = 0; d < 3; d++) {
      clo[d] = glo[d];
      chi_[d] = ghi[d];
    }
    for (int d = 0; d < 3; d++) {
      if (!p.present[d]) continue;
      for (int q = 0; q < 3; q++) {
        lo[q] = clo[q];
        hi[q] = chi_[q];
      }
      hi[d] = ilo[d] - 1;
      add_box(box_bnd, lo, hi, dim, fblock);
      lo[d] = ihi[d] + 1;
      hi[d] = chi_[d];
      add_box(box_bnd, lo, hi, dim, fblock);
      clo[d] = ilo[d];
      chi_[d] = ihi[d];
    }
    check_boxes(glo, ghi);
  }

  // every box must lie inside the point range 0..N-1 of each direction, and
  // the boxes must cover it exactly once
  // the 3-D launches must cover points 0..N-1 of every direction exactly once
  // and stay inside them (rows, x slabs, y slabs)
  void check_bands(const Plan &p) const {
    std::vector<unsigned char> seen((size_t)p.N[0] * p.N[1] * p.N[2], 0);
    auto mark = [&](int k0, int k1, int k2) {
      if (k0 < 0 || k0 >= p.N[0] || k1 < 0 || k1 >= p.N[1] || k2 < 0 || k2 >= p.N[2])
        throw Error("internal: launch band outside the grid");
      seen[((size_t)k0 * p.N[1] + k1) * p.N[2] + k2]++;
    };
    auto kof = [](const Span &s, int t) { return t + (t < s.split ? s.a0 : s.a1); };
    auto band = [&](const Band &b) {
      for (int t0 = 0; t0 < b.s[0].n; t0++)
        for (int t1 = 0; t1 < b.s[1].n; t1++)
          for (int t2 = 0; t2 < b.s[2].n; t2++)
            mark(kof(b.s[0], t0), kof(b.s[1], t1), kof(b.s[2], t2));
    };
    bool zi = false; // which shell: full-row faces or z-interior faces + z edges
    auto slabs = [&] {
      if (zi) {
        band(band_xface_zi);
        band(band_yface_zi);
        band(band_xzedge);
        band(band_yzedge);
      }
      else {
        band(band_xface);
        band(band_yface);
      }
      band(band_xyedge);
    };
    slabs();
    band(band_rows);
    for (unsigned char v : seen)
      if (v != 1) throw Error("internal: launch bands do not tile the grid");
    // the one-point core + z ends instead of the rows, with the FP64 shell
    for (int pass = 0; pass < 2; pass++) {
      zi = pass == 1;
      std::fill(seen.begin(), seen.end(), 0);
      slabs();
      if (band_core.s[2].n > 0) {
        band(band_core);
        band(band_zend);
      }
      else
        band(band_rows);
      for (unsigned char v : seen)
        if (v != 1) throw Error("internal: launch bands do not tile the grid");
    }
    zi = false;
    // the FP32 B update: core + z ends instead of the rows
    std::fill(seen.begin(), seen.end(), 0);
    slabs();
    band(band_zend);
    for (int t0 = 0; t0 < qcore.n[0]; t0++)
      for (int t1 = 0; t1 < qcore.n[1]; t1++)
        for (int k2 = qcore.lo[2]; k2 < qcore.zend; k2++)
          mark(qcore.lo[0] + t0, qcore.lo[1] + t1, k2);
    if (qcore.zend > qcore.lo[2] && (qcore.lo[2] % 4 || qcore.zend % 4 || qcore.lo[2] < 1 || qcore.zend > p.N[2]))
      throw Error("internal: quad core not aligned");
    for (unsigned char v : seen)
      if (v != 1) throw Error("internal: launch bands do not tile the grid");
  }

  void check_boxes(const int glo[3], const int ghi[3]) const {
    long long total = 1, covered = 0;
    for (int d = 0; d < 3; d++)
      total *= ghi[d] - glo[d] + 1;
    for (const BoxList *L : {&box_int, &box_bnd})
      for (int q = 0; q < L->n; q++) {
        long long v = 1;
        for (int d = 0; d < 3; d++) {
          if (L->lo[q][d] < glo[d] || L->lo[q][d] + L->ext[q][d] - 1 > ghi[d])
            throw Error("internal: launch box outside the grid");
          v *= L->ext[q][d];
        }
        covered += v;
      }
    if (covered != total) throw Error("internal: launch boxes do not tile the grid");
  }

  template <int DIM, int MASK>
  void fused_step_t(Plan &p, const DipoleVals &curb, const DipoleVals &curd, const DipoleVals &dip) {
    FusedArgs<R> a = fused_args(p, !has_b_current);
    const bool cndB = a.cnd[3][0] || a.cnd[3][1] || a.cnd[3][2];
    const bool cndD = a.cnd[2][0] || a.cnd[2][1] || a.cnd[2][2];
    const bool zp = a.pml[2] != 0;
    constexpr bool F32 = std::is_same<R, float>::value;
    if constexpr (DIM == 3) {
      fork();
      if constexpr (F32) {
        // the side streams' launches first (their blocks go first anyway)
        launch_b_band<false, false>(band_zend, a, cndB, zp, S(2));
        launch_b_qfaces(a, cndB, S(1));
        launch_b_shell(a, cndB, zp, S(0));
        const dim3 g = core_grid();
        if (g.x) {
          if (cndB) b3q_core_kernel<true><<<g, 256, 0, stream>>>(a, qcore);
          else b3q_core_kernel<false><<<g, 256, 0, stream>>>(a, qcore);
          nlaunch++;
        }
      }
      else if (band_core.s[2].n > 0) {
        launch_b_band<false, false, false>(band_core, a, cndB, zp, stream);
        launch_b_band<false, false>(band_zend, a, cndB, zp, S(2));
      }
      else
        launch_b_band<false, false>(band_rows, a, cndB, zp, stream);
      // the shell: x and y slab faces over their z interior (no z flags;
      // FP32: quads, a launch of their own) and their z ends, and the x-y
      // edges, one launch; the z ends of the rows beside them
      if (!F32) launch_b_shell_bands(a, cndB, zp);
      join();
    }
    else {
      if (box_int.n) {
        fused_b_kernel<R, DIM, MASK, true><<<box_int.blk0[box_int.n], fblock, 0, stream>>>(a, box_int);
        nlaunch++;
      }
      if (box_bnd.n) {
        fused_b_kernel<R, DIM, MASK, false><<<box_bnd.blk0[box_bnd.n], fblock, 0, stream>>>(a, box_bnd);
        nlaunch++;
      }
    }
    if (has_b_current) {
      step_current(p, MFD_B, curb);
      for (int d = 0; d < 3; d++)
        if (p.have[comp(MFD_H, d)]) update_h(p, comp(MFD_H, d));
    }
    join_samples(); // the previous step's E/D samples read what D/E writes
    bool dcur = false;
    for (int d = 0; d < 3; d++)
      dcur = dcur || ncur[comp(MFD_D, d)] > 0;
    if (dcur) {
      // current sources on D act between the curl and the E update: run the
      // generic D curl, the current kernel, then the fused kernel's E part is
      // not usable; fall back to the generic D/E sequence
      for (int d = 0; d < 3; d++)
        if (p.have[comp(MFD_D, d)]) curl(p, comp(MFD_D, d));
      step_current(p, MFD_D, curd);
      update_e(p, dip);
      return;
    }
    if constexpr (DIM == 3) {
      if (p.any_offdiag) {
        offdiag_de3(p, a, cndD, zp, dip);
        return;
      }
    }
    const bool e_only = DIM == 3 && src_e_only;
    for (int d = 0; d < 3; d++)
      if (nsrcpts[d] && !e_only) {
        fused_src_pre_kernel<R, DIM, MASK><<<(nsrcpts[d] + 127) / 128, 128, 0, stream>>>(
            a, d_srcpts[d], nsrcpts[d], d, dip, d_fsrcbuf[d]);
        nlaunch++;
      }
    if constexpr (DIM == 3) {
      if (e_only || !(nsrcpts[0] || nsrcpts[1] || nsrcpts[2])) {
        stream_order_kernel<<<1, 32, 0, stream>>>();
        nlaunch++;
      }
      fork();
      // the side streams' launches first (their blocks start at once).
      // D/E faces: with poles confined to one end of the z interior, its
      // pole-free part as quads and the rest in the shell
      bool split = false;
      if (F32 && use_qfaces && a.npoles > 0 && a.npoles <= 2 && pole_z1 >= 0) {
        const Span zi = band_xface_zi.s[2];
        const int zlo = zi.a0, zhi = zi.a0 + zi.n; // [zlo, zhi)
        const int p0 = std::max(zlo, pole_z0), p1 = std::min(zhi, pole_z1);
        Span zq{}, zs{};
        if (p1 <= p0) { // no pole in the z interior
          zq = zi;
          zs = span_run(0, -1);
          split = true;
        }
        else if (p0 == zlo && p1 < zhi) {
          zs = span_run(zlo, p1 - 1);
          zq = span_run(p1, zhi - 1);
          split = true;
        }
        else if (p1 == zhi && p0 > zlo) {
          zs = span_run(p0, zhi - 1);
          zq = span_run(zlo, p0 - 1);
          split = true;
        }
        if (split && zq.n % 4 == 0 && zq.a0 % 4 == 0) {
          if (!qf_am_done) {
            Band f0 = band_xface_zi, f1 = band_yface_zi;
            f0.s[2] = f1.s[2] = zq;
            qf_am = uniform_am({f0, f1});
            qf_am_done = true;
          }
          FusedArgs<R> aq = a;
          aq.am_all = qf_am;
          launch_de_qfaces(aq, cndD, S(1), &zq);
          launch_de_shell_split(a, cndD, zp, &zs);
        }
        else
          split = false;
      }
      if (!split && F32) {
        const bool qde = launch_de_qfaces(a, cndD, S(1));
        launch_de_shell(a, cndD, zp, qde, S(0));
      }
      else if (!split)
        launch_de_shell_bands(a, cndD, zp);
      // FP64 (issue-bound): the flagless core and the z ends; FP32
      // (bandwidth-bound): whole rows, whose z slabs ride along in full warps
      if (!F32 && band_core.s[2].n > 0) {
        launch_de_band<false, false>(band_zend, a, cndD, zp, S(2));
        launch_de_band<false, false, false>(band_core, a, cndD, zp, stream);
      }
      else if (a.npoles > 0 && pole_z1 >= 0 && (pole_z0 > 0 || std::min(pole_z1, p.N[2]) < p.N[2])) {
        // rows (z points 0..N-1) split along z at the pole region: the kernel
        // with poles in registers where some pole is active, the pole-free one
        // elsewhere (P stays 0 there; its registers would only cost occupancy)
        const int z1 = std::min(pole_z1, p.N[2]);
        Band bn = band_rows;
        bn.s[2] = z1 > pole_z0 ? span_outside(p.N[2], pole_z0, z1 - 1) : span_run(0, p.N[2] - 1);
        dim3 g, blk;
        band_shape(bn, g, blk);
        if (g.x) {
          if (!bn_am_done) {
            bn_am = uniform_am({bn});
            bn_am_done = true;
          }
          FusedArgs<R> an = a;
          an.am_all = bn_am;
          launch_de_band_p<false, false, 0>(bn, g, blk, an, cndD, zp, S(2));
          nlaunch++;
        }
        if (z1 > pole_z0) {
          Band bp = band_rows;
          bp.s[2] = span_run(pole_z0, z1 - 1);
          // the pole rows: their segments' activity word as a parameter
          // when it is the same everywhere there
          if (!bp_am_done) {
            bp_am = uniform_am({bp});
            bp_am_done = true;
          }
          FusedArgs<R> ab = a;
          ab.am_all = bp_am;
          launch_de_band<false, false>(bp, ab, cndD, zp, stream);
        }
      }
      else
        launch_de_band<false, false>(band_rows, a, cndD, zp, stream);
      join();
    }
    else {
      if (box_int.n) {
        fused_de_kernel<R, DIM, MASK, true><<<box_int.blk0[box_int.n], fblock, 0, stream>>>(a, box_int);
        nlaunch++;
      }
      if (box_bnd.n) {
        fused_de_kernel<R, DIM, MASK, false><<<box_bnd.blk0[box_bnd.n], fblock, 0, stream>>>(a, box_bnd);
        nlaunch++;
      }
    }
    for (int d = 0; d < 3; d++)
      if (nsrcpts[d]) {
        if (e_only)
          src_e_kernel<R><<<(nsrcpts[d] + 127) / 128, 128, 0, stream>>>(a.e[d], a.d[d], a.chi[d], d_srcpts[d],
                                                                         nsrcpts[d], dip);
        else
          fused_src_post_kernel<R, DIM, MASK><<<(nsrcpts[d] + 127) / 128, 128, 0, stream>>>(
              a, d_srcpts[d], nsrcpts[d], d, d_fsrcbuf[d]);
        nlaunch++;
      }
  }

  // The 3-D step as one CUDA graph, captured at the first step: the side
  // streams' forks and joins become graph edges; the main stream waits for
  // the previous step's E/D samples before the launch.  Each step sets its
  // source values on the source kernels' nodes.  Steps with current sources
  // or off-diagonal chi1inv, or integrated sources that need the kernels
  // around the D/E launches, keep the stream launches, and so do steps with
  // Lorentz/Drude poles: on GB300 the graph took the 256^3 step without
  // poles 5 us faster, the 384^2 x 192 step with poles (rows split at the
  // pole region) 4 us slower, its side-stream kernels finishing after the
  // main-stream ones instead of under them.
  cudaGraph_t sgraph = nullptr;
  cudaGraphExec_t sgexec = nullptr;
  struct SrcNode {
    cudaGraphNode_t node;
    cudaKernelNodeParams kp;
    R *e;
    const R *d, *chi;
    const SrcPoint *pts;
    int n;
  };
  std::vector<SrcNode> src_nodes;
  long long graph_nlaunch = 0;
  bool graph_off = false, capturing = false;
  bool graph_eligible(const Plan &p) const {
    if (fused_mask != MASK3 || has_b_current || p.any_offdiag || !poles.empty()) return false;
    for (int d = 0; d < 3; d++)
      if (ncur[comp(MFD_D, d)] > 0 || (nsrcpts[d] > 0 && !src_e_only)) return false;
    return true;
  }
  bool graph_step(Plan &p, const DipoleVals &curb, const DipoleVals &curd, const DipoleVals &dip) {
    if (graph_off || !graph_eligible(p)) return false;
    // the previous step's E/D samples finish before the graph starts (the
    // graph holds no wait on them)
    join_samples();
    if (!sgexec) {
      // capture (the side streams join it through the fork events)
      fork_from = nullptr;
      const long long l0 = nlaunch;
      cuda_check(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "begin capture");
      capturing = true;
      bool ok = true;
      try {
        fused_step_t<3, MASK3>(p, curb, curd, dip);
      } catch (const Error &) {
        ok = false;
      }
      capturing = false;
      ok = cudaStreamEndCapture(stream, &sgraph) == cudaSuccess && ok;
      ok = ok && cudaGraphInstantiate(&sgexec, sgraph, 0) == cudaSuccess;
      nlaunch = l0;
      graph_nlaunch = 0;
      if (!ok) {
        // not capturable here: the stream launches from now on
        (void)cudaGetLastError();
        if (sgexec) cudaGraphExecDestroy(sgexec);
        if (sgraph) cudaGraphDestroy(sgraph);
        sgexec = nullptr;
        sgraph = nullptr;
        graph_off = true;
        return false;
      }
      size_t nn = 0;
      cuda_check(cudaGraphGetNodes(sgraph, nullptr, &nn), "graph nodes");
      std::vector<cudaGraphNode_t> nodes(nn);
      cuda_check(cudaGraphGetNodes(sgraph, nodes.data(), &nn), "graph nodes");
      for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType ty;
        cuda_check(cudaGraphNodeGetType(nd, &ty), "graph node type");
        if (ty != cudaGraphNodeTypeKernel) continue;
        SrcNode sn{};
        cuda_check(cudaGraphKernelNodeGetParams(nd, &sn.kp), "graph node params");
        graph_nlaunch++;
        if (sn.kp.func != (void *)src_e_kernel<R>) continue;
        sn.node = nd;
        sn.e = *(R **)sn.kp.kernelParams[0];
        sn.d = *(const R **)sn.kp.kernelParams[1];
        sn.chi = *(const R **)sn.kp.kernelParams[2];
        sn.pts = *(const SrcPoint **)sn.kp.kernelParams[3];
        sn.n = *(int *)sn.kp.kernelParams[4];
        src_nodes.push_back(sn);
      }
    }
    for (SrcNode &sn : src_nodes) {
      DipoleVals dv = dip;
      void *args[] = {&sn.e, &sn.d, &sn.chi, &sn.pts, &sn.n, &dv};
      cudaKernelNodeParams kp = sn.kp;
      kp.kernelParams = args;
      kp.extra = nullptr;
      cuda_check(cudaGraphExecKernelNodeSetParams(sgexec, sn.node, &kp), "source node values");
    }
    cuda_check(cudaGraphLaunch(sgexec, stream), "graph launch");
    nlaunch += graph_nlaunch;
    return true;
  }

  void fused_step(Plan &p, const DipoleVals &curb, const DipoleVals &curd, const DipoleVals &dip) {
    if (graph_step(p, curb, curd, dip)) return;
    switch (fused_mask) {
      case MASK3: fused_step_t<3, MASK3>(p, curb, curd, dip); break;
      case MASK_TM: fused_step_t<2, MASK_TM>(p, curb, curd, dip); break;
      case MASK_TE: fused_step_t<2, MASK_TE>(p, curb, curd, dip); break;
      case MASK_1D: fused_step_t<1, MASK_1D>(p, curb, curd, dip); break;
      default: throw Error("no fused kernel for this component set");
    }
  }

  void setup_sources(Plan &p) {
    if (p.srcs.size() > 16) throw Error("at most 16 source time functions are supported");
    // integrated E sources grouped per (component, point), in list order
    bool e_only = p.g.dim == 3 && !p.any_offdiag;
    for (int d = 0; d < 3; d++) {
      std::vector<SrcPoint> pts;
      std::vector<int64_t> keys;
      for (const SourceGroup &sg : p.sources) {
        if (sg.c != comp(MFD_E, d) || !p.srcs[sg.src].integrated) continue;
        for (size_t j = 0; j < sg.idx.size(); j++) {
          int64_t di = sg.idx[j];
          size_t q = std::find(keys.begin(), keys.end(), di) - keys.begin();
          if (q == keys.size()) {
            keys.push_back(di);
            SrcPoint sp{};
            sp.i = p.store_index_of_dense(di);
            p.dense_coords(di, sp.k);
            pts.push_back(sp);
          }
          SrcPoint &sp = pts[q];
          if (sp.nterm >= MAXS) throw Error("too many sources on one point");
          sp.src[sp.nterm] = sg.src;
          sp.amp[sp.nterm][0] = sg.amp[j].real();
          sp.amp[sp.nterm][1] = sg.amp[j].imag();
          sp.nterm++;
        }
      }
      // points outside the updated range are never advanced (metal walls);
      // with off-diagonal chi1inv their f_minus_p is still read by the
      // neighbouring E points, so they stay (only f_minus_p uses the list then)
      std::vector<SrcPoint> keep;
      int ec = comp(MFD_E, d);
      for (size_t q0 = 0; q0 < pts.size(); q0++) {
        const SrcPoint &sp = pts[q0];
        bool in = true;
        for (int q = 0; q < 3; q++)
          in = in && sp.k[q] >= p.klo[ec][q] && sp.k[q] <= p.khi[ec][q];
        if (!(in || p.any_offdiag)) continue;
        keep.push_back(sp);
        // E_d sits at half-pixel 2k + 1 along d; its f_w slab there
        const int pw = 2 * sp.k[d] + 1;
        if (p.pml_dir[d] && ((p.T[d][0] > 0 && pw <= 2 * p.T[d][0]) || (p.T[d][1] > 0 && pw > 2 * (p.N[d] - p.T[d][1]))))
          e_only = false;
        for (const Pole &pl : p.poles)
          if (!pl.sigma[d].empty() && pl.sigma[d][keys[q0]] != 0.0) e_only = false;
      }
      nsrcpts[d] = (int)keep.size();
      if (!keep.empty()) {
        d_srcpts[d] = dupload(keep);
        d_srcbuf[d] = dalloc<EPoint<R>>(keep.size());
        d_fsrcbuf[d] = dalloc<DEOut<R>>(keep.size());
      }
    }
    src_e_only = e_only;
    // current sources (non-integrated) on D or B
    for (int c = 0; c < NC; c++) {
      int t = ctype(c);
      if (t != MFD_D && t != MFD_B) continue;
      std::vector<CurPoint> pts;
      int srct = t == MFD_D ? MFD_E : MFD_H;
      for (const SourceGroup &sg : p.sources) {
        if (sg.c != comp(srct, cdir(c)) || p.srcs[sg.src].integrated) continue;
        for (size_t j = 0; j < sg.idx.size(); j++) {
          CurPoint cp{};
          cp.i = p.store_index_of_dense(sg.idx[j]);
          cp.src = sg.src;
          cp.amp[0] = sg.amp[j].real();
          cp.amp[1] = sg.amp[j].imag();
          pts.push_back(cp);
        }
      }
      ncur[c] = (int)pts.size();
      if (!pts.empty()) d_cur[c] = dupload(pts);
    }
  }

  void add_monitor(Plan &p, int id) override {
    join_dft();
    if ((int)mons.size() <= id) mons.resize(id + 1);
    const Monitor &m = p.monitors[id];
    DMon &dm = mons[id];
    bump(id);
    dm.acc = dzeros<double2>(m.npts * m.freq.size());
    dm.ph = dalloc<double2>(m.freq.size());
    dm.freq = dupload(m.freq);
    for (int d = 0; d < 3; d++)
      if (!m.w[d].empty()) dm.w[d] = dupload(m.w[d]);
    dm.block = sizeof(R) == 4 && !getenv("MFD_DIRECT_DFT") && !p.complex_fields;
    // the block contraction on the tensor cores unless MFD_DFT_CUDA_CORES is
    // set (the CUDA-core kernel stays as the cross-check)
    dm.tc = dm.block && !getenv("MFD_DFT_CUDA_CORES");
    if (dm.tc && !d_tc_err) {
      d_tc_err = dzeros<int>(1);
      cuda_check(cudaFuncSetAttribute(dft_contract_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM),
                 "tensor-core DFT shared memory");
    }
    const int t = ctype(m.c);
    dm.async = fused_mask == MASK3 && (t == MFD_E || t == MFD_D);
    if (dm.block) {
      dm.Ab[0] = dm.A = dalloc<float>((size_t)DFT_BLOCK_T * m.npts);
      dm.B = dalloc<float2>((size_t)DFT_BLOCK_T * m.freq.size());
      if (dm.async) {
        dm.Ab[1] = dalloc<float>((size_t)DFT_BLOCK_T * m.npts);
        for (cudaEvent_t &e : dm.fdone)
          cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
      }
    }
    cuda_check(cudaStreamSynchronize(stream), "monitor sync");
  }

  // contract the samples of the current block into the running sums
  void dft_flush(Plan &p, int id) {
    join_dft();
    flush_on(p, id, stream);
  }
  void flush_on(Plan &p, int id, cudaStream_t st) {
    const Monitor &m = p.monitors[id];
    DMon &dm = mons[id];
    if (!dm.block || dm.cnt == 0) return;
    const int nf = (int)m.freq.size();
    const int half = (ctype(m.c) == MFD_H || ctype(m.c) == MFD_B) ? 1 : 0;
    dft_block_phase_kernel<<<dim3((nf + 127) / 128, dm.cnt), 128, 0, st>>>(
        dm.freq, nf, dm.cnt, dm.tn0, m.decimation, p.dt, half, m.scale.real(), m.scale.imag(), dm.B);
    const int chunk = 64; // frequencies per shared-memory pass (<= 32 KB)
    size_t smem = (size_t)dm.cnt * chunk * sizeof(float2);
    long long np = (long long)m.npts;
    if (dm.tc)
      dft_contract_tc_kernel<<<(unsigned)((np + TC_M - 1) / TC_M), TC_THREADS, TC_SMEM, st>>>(dm.A, dm.cnt, np, dm.B,
                                                                                              nf, dm.acc, d_tc_err);
    else
      dft_contract_kernel<<<(unsigned)((np + 127) / 128), 128, smem, st>>>(dm.A, dm.cnt, np, dm.B, nf, dm.acc);
    nlaunch += 2;
    dm.cnt = 0;
    if (dm.async) {
      // the next samples go to the other staging block once its own
      // contraction is done
      cuda_check(cudaEventRecord(dm.fdone[dm.cur], st), "event record");
      dm.issued[dm.cur] = true;
      dm.cur ^= 1;
      dm.A = dm.Ab[dm.cur];
    }
  }

  Box full_box(const Plan &p, int c) const {
    Box b;
    for (int d = 0; d < 3; d++) {
      b.lo[d] = p.klo[c][d];
      b.n[d] = p.khi[c][d] - p.klo[c][d] + 1;
    }
    return b;
  }

  void launch_dims(const Box &b, dim3 &grid, dim3 &block) const {
    int nf = b.n[geo.fast], nm = b.n[geo.mid], ns = b.n[geo.slow];
    int bx = nf >= 128 ? 128 : (nf >= 64 ? 64 : 32);
    int by = 256 / bx;
    block = dim3(bx, by, 1);
    grid = dim3((nf + bx - 1) / bx, (nm + by - 1) / by, ns);
  }
  bool box_empty(const Box &b) const { return b.n[0] <= 0 || b.n[1] <= 0 || b.n[2] <= 0; }

  void curl(Plan &p, int c) {
    const Plan::Curl &cp = p.curl[c];
    if (cp.g1 < 0) return;
    CurlArgs<R> a{};
    a.f = f[c];
    a.fu = fu[c];
    a.fcnd = fcnd[c];
    a.cnd = cnd[c];
    a.cndinv = cndinv[c];
    bool dcurl = ctype(c) == MFD_D;
    auto src_ptrs = [&](int gc, const R *&gp, const R *&gh, int &gdir) {
      gdir = cdir(gc);
      if (dcurl) {
        gp = f[comp(MFD_B, gdir)];
        gh = p.pml_dir[gdir] ? f[gc] : nullptr;
      }
      else {
        gp = f[gc];
        gh = nullptr;
      }
    };
    src_ptrs(cp.g1, a.g1, a.g1h, a.g1dir);
    if (cp.g2 >= 0) src_ptrs(cp.g2, a.g2, a.g2h, a.g2dir);
    a.s1 = cp.s1;
    a.s2 = cp.s2;
    a.dtdx = cp.flip ? -R(p.g.courant) : R(p.g.courant);
    a.dt2 = R(p.dt) * R(0.5);
    a.dsig = cp.dsig;
    a.dsigu = cp.dsigu;
    for (int d = 0; d < 3; d++)
      a.shift[d] = p.shift[c][d];
    a.cond_chunks = 0;
    if (!p.cond_chunk[c].empty())
      for (int r = 0; r < 27; r++)
        if (p.cond_chunk[c][r]) a.cond_chunks |= 1u << r;
    a.box = full_box(p, c);
    if (box_empty(a.box)) return;
    dim3 grid, block;
    launch_dims(a.box, grid, block);
    curl_kernel<R><<<grid, block, 0, stream>>>(geo, tb, a);
    nlaunch++;
  }

  void update_h(Plan &p, int hc) {
    int d = cdir(hc);
    if (!p.pml_dir[d]) return;
    HArgs<R> a{};
    a.h = f[hc];
    a.fw = fw[hc];
    a.b = f[comp(MFD_B, d)];
    a.dir = d;
    for (int q = 0; q < 3; q++)
      a.shift[q] = p.shift[hc][q];
    Box full = full_box(p, hc);
    // the two slabs along d: positions 2k <= 2T_lo and 2k > 2(N - T_hi)
    for (int side = 0; side < 2; side++) {
      if (p.T[d][side] == 0) continue;
      Box b = full;
      int lo = full.lo[d], hi = full.lo[d] + full.n[d] - 1;
      if (side == 0) hi = std::min(hi, p.T[d][0]);
      else lo = std::max(lo, p.N[d] - p.T[d][1] + 1);
      b.lo[d] = lo;
      b.n[d] = hi - lo + 1;
      if (box_empty(b)) continue;
      a.box = b;
      dim3 grid, block;
      launch_dims(b, grid, block);
      h_pml_kernel<R><<<grid, block, 0, stream>>>(geo, tb, a);
      nlaunch++;
    }
  }

  EArgs<R> eargs(Plan &p, int d) {
    int ec = comp(MFD_E, d);
    EArgs<R> a{};
    a.e = f[ec];
    a.fw = fw[ec];
    a.dfield = f[comp(MFD_D, d)];
    a.chi = chi[ec];
    a.dir = d;
    for (int q = 0; q < 3; q++)
      a.shift[q] = p.shift[ec][q];
    a.npoles = (int)poles.size();
    for (int q = 0; q < a.npoles; q++) {
      a.pole[q].P = poles[q].P[d];
      a.pole[q].PP = poles[q].PP[d];
      a.pole[q].s = poles[q].s[d];
      a.pole[q].gamma1inv = poles[q].gamma1inv;
      a.pole[q].gamma1 = poles[q].gamma1;
      a.pole[q].w0 = poles[q].w0;
      a.pole[q].w0d = poles[q].w0d;
    }
    a.box = full_box(p, ec);
    return a;
  }

  // E from f_minus_p of all D components (off-diagonal chi1inv): f_minus_p
  // first, then every E component with its OFFDIAG terms and poles
  void update_e_offdiag(Plan &p, const DipoleVals &dip) {
    for (int d = 0; d < 3; d++) {
      if (!fmp[d]) continue;
      FmpArgs<R> fa{};
      fa.out = fmp[d];
      fa.d = f[comp(MFD_D, d)];
      fa.np = (int)poles.size();
      for (int q = 0; q < fa.np; q++)
        fa.p[q] = poles[q].P[d];
      fa.n = p.nstore;
      fmp_kernel<R><<<(unsigned)((p.nstore + 255) / 256), 256, 0, stream>>>(fa);
      nlaunch++;
      if (nsrcpts[d]) {
        src_fmp_kernel<R><<<(nsrcpts[d] + 127) / 128, 128, 0, stream>>>(fa, d_srcpts[d], nsrcpts[d], dip);
        nlaunch++;
      }
    }
    for (int d = 0; d < 3; d++) {
      int ec = comp(MFD_E, d);
      if (!p.have[ec]) continue;
      EArgs<R> a = eargs(p, d);
      if (box_empty(a.box)) continue;
      if (fmp[d]) {
        a.dfield = fmp[d];
        a.pre = 1;
      }
      a.noff = p.offdiag[d].n;
      a.s = (long long)p.stride[d];
      for (int q = 0; q < a.noff; q++) {
        const int od = p.offdiag[d].dir[q];
        a.og[q] = fmp[od] ? fmp[od] : f[comp(MFD_D, od)];
        a.ou[q] = chioff[d][q];
        a.so[q] = (long long)p.stride[od];
      }
      dim3 grid, block;
      launch_dims(a.box, grid, block);
      e_kernel<R><<<grid, block, 0, stream>>>(geo, tb, a);
      nlaunch++;
    }
  }

  void update_e(Plan &p, const DipoleVals &dip) {
    if (p.any_offdiag) {
      update_e_offdiag(p, dip);
      return;
    }
    for (int d = 0; d < 3; d++) {
      int ec = comp(MFD_E, d);
      if (!p.have[ec]) continue;
      EArgs<R> a = eargs(p, d);
      if (box_empty(a.box)) continue;
      int ns = nsrcpts[d];
      if (ns) {
        src_pre_kernel<R><<<(ns + 127) / 128, 128, 0, stream>>>(geo, tb, a, d_srcpts[d], ns, dip,
                                                               d_srcbuf[d]);
        nlaunch++;
      }
      dim3 grid, block;
      launch_dims(a.box, grid, block);
      e_kernel<R><<<grid, block, 0, stream>>>(geo, tb, a);
      nlaunch++;
      if (ns) {
        src_post_kernel<R><<<(ns + 127) / 128, 128, 0, stream>>>(geo, a, d_srcpts[d], ns, d_srcbuf[d]);
        nlaunch++;
      }
    }
  }

  void step_current(Plan &p, int ft, const DipoleVals &cur) {
    for (int d = 0; d < 3; d++) {
      int c = comp(ft, d);
      if (!ncur[c]) continue;
      src_current_kernel<R><<<(ncur[c] + 127) / 128, 128, 0, stream>>>(f[c], cndinv[c], d_cur[c],
                                                                       ncur[c], cur, p.dt);
      nlaunch++;
    }
  }

  // E/D monitors of the 3-D step: sampled on dstream once the step's main
  // stream work is queued (launch_samples)
  struct QueuedSample {
    int id;
    double time;
    int64_t tn;
  };
  std::vector<QueuedSample> queued;
  void dft(Plan &p, int id, double time, int64_t tn) {
    bump(id);
    if (mons[id].async) queued.push_back({id, time, tn});
    else dft_launch(p, id, time, tn, stream);
  }
  void launch_samples(Plan &p) {
    if (queued.empty()) return;
    cuda_check(cudaEventRecord(dft_in_ev, stream), "event record");
    cuda_check(cudaStreamWaitEvent(dstream, dft_in_ev, 0), "stream wait");
    dft_pending = true;
    for (const QueuedSample &q : queued)
      dft_launch(p, q.id, q.time, q.tn, dstream);
    queued.clear();
    if (!sgexec) {
      // the next fork waits on the same event as the samples (nothing is
      // queued on the main stream behind it before then; every other call
      // joins first)
      fork_from = dft_in_ev;
    }
  }
  void dft_launch(Plan &p, int id, double time, int64_t tn, cudaStream_t st) {
    const Monitor &m = p.monitors[id];
    DMon &dm = mons[id];
    int nf = (int)m.freq.size();
    DftArgs<R> a{};
    a.f = f[m.c];
    a.fb = nullptr;
    a.fim = cplx ? fim[m.c] : nullptr;
    a.fbim = nullptr;
    if (ctype(m.c) == MFD_H) {
      int d = cdir(m.c);
      a.hdir = d;
      a.hshift = p.shift[m.c][d];
      a.fb = f[comp(MFD_B, d)];
      if (!p.pml_dir[d]) a.f = a.fb;
      if (cplx) {
        a.fbim = fim[comp(MFD_B, d)];
        if (!p.pml_dir[d]) a.fim = a.fbim;
      }
    }
    for (int d = 0; d < 3; d++) {
      a.w[d] = dm.w[d];
      a.lo[d] = m.lo[d];
      a.n[d] = m.hi[d] - m.lo[d] + 1;
    }
    a.dV = m.dV;
    a.include_weights = m.include_weights;
    a.sqrt_w = m.sqrt_weights;
    a.dim = p.g.dim;
    a.ad0 = a.ad1 = -1;
    if (m.centered)
      for (int d = 0; d < 3; d++)
        if (p.present[d] && p.shift[m.c][d] == 0) {
          if (a.ad0 >= 0) a.ad1 = d;
          else a.ad0 = d;
        }
    a.acc = dm.acc;
    a.ph = dm.ph;
    a.nf = nf;
    a.npts = (long long)m.npts;
    if (dm.block) {
      if (dm.cnt == 0) {
        dm.tn0 = tn;
        if (dm.async && dm.issued[dm.cur]) {
          cuda_check(cudaStreamWaitEvent(dstream, dm.fdone[dm.cur], 0), "stream wait");
          dm.issued[dm.cur] = false;
        }
      }
      dft_sample_kernel<R><<<(unsigned)((a.npts + 255) / 256), 256, 0, st>>>(geo, a, dm.A + (size_t)dm.cnt * m.npts);
      nlaunch++;
      if (++dm.cnt == DFT_BLOCK_T) {
        if (dm.async) {
          cuda_check(cudaEventRecord(fl_in_ev, dstream), "event record");
          cuda_check(cudaStreamWaitEvent(fstream, fl_in_ev, 0), "stream wait");
          flush_on(p, id, fstream);
          fl_pending = true;
        }
        else
          dft_flush(p, id);
      }
      return;
    }
    dft_phase_kernel<<<(nf + 127) / 128, 128, 0, st>>>(dm.freq, nf, time, m.scale.real(), m.scale.imag(), dm.ph);
    nlaunch++;
    long long total = a.npts * nf;
    int bs = 256;
    long long nb = (total + bs - 1) / bs;
    dft_kernel<R><<<(unsigned)nb, bs, 0, st>>>(geo, a);
    nlaunch++;
  }

  void step(Plan &p, int64_t t, const std::vector<SrcStepValues> &vals) override {
    DipoleVals curb{}, curd{}, dip{};
    for (size_t k = 0; k < vals.size() && k < 16; k++) {
      curb.re[k] = vals[k].cur_b.real();
      curb.im[k] = vals[k].cur_b.imag();
      curd.re[k] = vals[k].cur_d.real();
      curd.im[k] = vals[k].cur_d.imag();
      dip.re[k] = vals[k].dip_e.real();
      dip.im[k] = vals[k].dip_e.imag();
    }
    check_finite();
    if (fused_mask >= 0) fused_step(p, curb, curd, dip);
    else {
      // per part (real, then imaginary for complex fields): the B half-step,
      // its boundaries; then the D/E half-step, its boundaries
      const int nparts = cplx ? 2 : 1;
      for (int part = 0; part < nparts; part++) {
        if (part) swap_parts();
        for (int d = 0; d < 3; d++)
          if (p.have[comp(MFD_B, d)]) curl(p, comp(MFD_B, d));
        step_current(p, MFD_B, part ? imag_part(curb) : curb);
        for (int d = 0; d < 3; d++)
          if (p.have[comp(MFD_H, d)]) update_h(p, comp(MFD_H, d));
        if (part) swap_parts();
      }
      ghost_copy(p, MFD_B, MFD_H);
      for (int part = 0; part < nparts; part++) {
        if (part) swap_parts();
        for (int d = 0; d < 3; d++)
          if (p.have[comp(MFD_D, d)]) curl(p, comp(MFD_D, d));
        step_current(p, MFD_D, part ? imag_part(curd) : curd);
        if (!p.any_offdiag) update_e(p, part ? imag_part(dip) : dip);
        if (part) swap_parts();
      }
      if (p.any_offdiag) {
        // the off-diagonal terms read D (and P) at the not-owned points:
        // fill them first, as the reference's D boundary step does
        ghost_copy(p, MFD_D, MFD_D);
        for (int part = 0; part < nparts; part++) {
          if (part) swap_parts();
          update_e(p, part ? imag_part(dip) : dip);
          if (part) swap_parts();
        }
        ghost_copy_pols(p);
      }
      ghost_copy(p, MFD_D, MFD_E);
    }
    int64_t tn = t + 1;
    for (size_t id = 0; id < p.monitors.size() && !skip_dft; id++) {
      const Monitor &m = p.monitors[id];
      if (tn % m.decimation != 0) continue;
      double timeE = tn * p.dt;
      double time = (ctype(m.c) == MFD_H || ctype(m.c) == MFD_B) ? timeE - 0.5 * p.dt : timeE;
      dft(p, (int)id, time, tn);
    }
    if (finite_every > 0 && tn % finite_every == 0) launch_finite_probe(p);
    launch_samples(p);
  }

  // a batch of steps without a divergence probe returns once it is queued
  // (its device time is taken when asked for, the tensor-core error flag
  // where results are read); a batch with a probe waits for it, so that a
  // divergence raises in the call whose steps the probe saw
  bool probe_pending = false;
  void begin_steps() override {
    ms_pending = false; // the previous batch's time is not asked for any more
    cuda_check(cudaEventRecord(ev0, stream), "event record");
  }
  void end_steps() override {
    join_dft();
    cuda_check(cudaEventRecord(ev1, stream), "event record");
    cuda_check(cudaGetLastError(), "kernel launch");
    ms_pending = true;
    if (probe_pending) {
      cuda_check(cudaEventSynchronize(ev1), "event sync");
      probe_pending = false;
      last_step_ms();
      check_tc();
    }
    check_finite();
  }
  mutable bool ms_pending = false;
  double last_step_ms() const override {
    if (ms_pending) {
      float fms = 0;
      if (cudaEventSynchronize(ev1) != cudaSuccess || cudaEventElapsedTime(&fms, ev0, ev1) != cudaSuccess) return -1.0;
      ms = fms;
      ms_pending = false;
    }
    return ms;
  }
  long long launches() const override { return nlaunch; }
  void synchronize() override {
    join_dft();
    cuda_check(cudaStreamSynchronize(stream), "sync");
    check_finite();
  }

  // ------------------------------------------------------------ adjoint
  std::vector<int> dcomps;       // design E components
  Box dbox{};                    // design point box
  long long dnpts = 0;
  R *rec = nullptr;              // [slots][ncomp][dnpts]
  long long rec_slots = 0;
  std::vector<std::pair<void *, size_t>> state_list; // (pointer, bytes) of every state array
  std::vector<char *> snaps;
  R *lam_f[NC] = {}, *lam_fu[NC] = {}, *lam_fw[NC] = {}, *xbar[NC] = {};
  double *grad = nullptr;
  std::vector<double2 *> adj_G; // per monitor (null when the monitor has no gradient)
  bool skip_dft = false;

  void set_skip_dft(bool s) override { skip_dft = s; }

  void set_design(Plan &p, const std::vector<int> &comps, const int lo[3], const int hi[3]) override {
    join_dft();
    for (int c : comps)
      if (ctype(c) != MFD_E || !p.have[c]) throw Error("design components must be allocated E components");
    if (!p.poles.empty()) throw Error("the adjoint does not support dispersive materials yet");
    p.plan_offdiag();
    if (p.any_offdiag) throw Error("the adjoint does not support off-diagonal chi1inv yet");
    for (int c = 0; c < NC; c++)
      if (!p.cond[c].empty()) throw Error("the adjoint does not support conductivity yet");
    dcomps = comps;
    dnpts = 1;
    for (int d = 0; d < 3; d++) {
      if (lo[d] < 0 || hi[d] >= p.ext[d] || hi[d] < lo[d]) throw Error("design box out of range");
      dbox.lo[d] = lo[d];
      dbox.n[d] = hi[d] - lo[d] + 1;
      dnpts *= dbox.n[d];
    }
    // integrated sources inside the design box would make dE/dchi1inv = D - source
    for (const SourceGroup &sg : p.sources)
      for (int64_t di : sg.idx) {
        int k[3];
        p.dense_coords(di, k);
        bool in = true;
        for (int d = 0; d < 3; d++)
          in = in && k[d] >= dbox.lo[d] && k[d] < dbox.lo[d] + dbox.n[d];
        if (in && ctype(sg.c) == MFD_E) throw Error("a source lies inside the design region");
      }
  }

  void alloc_record(Plan &p, int64_t nslots) override {
    join_dft();
    (void)p;
    if (nslots <= rec_slots) return;
    rec = dalloc<R>((size_t)nslots * dcomps.size() * dnpts);
    rec_slots = nslots;
  }

  void record_design(Plan &p, int64_t slot) override {
    join_dft();
    for (size_t q = 0; q < dcomps.size(); q++) {
      int dc = comp(MFD_D, cdir(dcomps[q]));
      dim3 grid, block;
      launch_dims(dbox, grid, block);
      box_copy_kernel<R><<<grid, block, 0, stream>>>(geo, f[dc], rec + ((size_t)slot * dcomps.size() + q) * dnpts,
                                                      dbox);
      nlaunch++;
    }
    (void)p;
  }

  void collect_state(Plan &p) {
    if (!state_list.empty()) return;
    size_t bytes = p.nstore * sizeof(R);
    for (int c = 0; c < NC; c++) {
      for (R *ptr : {f[c], fu[c], fw[c], fcnd[c]})
        if (ptr) state_list.push_back({ptr, bytes});
    }
    for (auto &pl : poles)
      for (int d = 0; d < 3; d++)
        for (R *ptr : {pl.P[d], pl.PP[d]})
          if (ptr) state_list.push_back({ptr, bytes});
  }

  int snapshot(Plan &p) override {
    join_dft();
    collect_state(p);
    size_t tot = 0;
    for (auto &s_ : state_list)
      tot += s_.second;
    char *buf = dalloc<char>(tot);
    size_t off = 0;
    for (auto &s_ : state_list) {
      cuda_check(cudaMemcpyAsync(buf + off, s_.first, s_.second, cudaMemcpyDeviceToDevice, stream), "snapshot");
      off += s_.second;
    }
    snaps.push_back(buf);
    return (int)snaps.size() - 1;
  }

  void restore(Plan &p, int slot) override {
    join_dft();
    collect_state(p);
    size_t off = 0;
    for (auto &s_ : state_list) {
      cuda_check(cudaMemcpyAsync(s_.first, snaps[slot] + off, s_.second, cudaMemcpyDeviceToDevice, stream),
                 "restore");
      off += s_.second;
    }
  }

  void adjoint_begin(Plan &p, int nmon, const int *ids, const double *const *grads) override {
    join_dft();
    for (int c = 0; c < NC; c++) {
      if (!p.have[c]) continue;
      if (!lam_f[c]) lam_f[c] = dalloc<R>(p.nstore);
      cuda_check(cudaMemsetAsync(lam_f[c], 0, p.nstore * sizeof(R), stream), "memset");
      int t = ctype(c);
      if ((t == MFD_D || t == MFD_B) && fu[c]) {
        if (!lam_fu[c]) lam_fu[c] = dalloc<R>(p.nstore);
        cuda_check(cudaMemsetAsync(lam_fu[c], 0, p.nstore * sizeof(R), stream), "memset");
      }
      if ((t == MFD_E || t == MFD_H) && fw[c]) {
        if (!lam_fw[c]) lam_fw[c] = dalloc<R>(p.nstore);
        cuda_check(cudaMemsetAsync(lam_fw[c], 0, p.nstore * sizeof(R), stream), "memset");
      }
      if ((t == MFD_D || t == MFD_B) && !xbar[c]) xbar[c] = dalloc<R>(p.nstore);
      if (xbar[c]) cuda_check(cudaMemsetAsync(xbar[c], 0, p.nstore * sizeof(R), stream), "memset");
    }
    if (!grad) grad = dalloc<double>(std::max<size_t>(1, dcomps.size() * dnpts));
    cuda_check(cudaMemsetAsync(grad, 0, std::max<size_t>(1, dcomps.size() * dnpts) * sizeof(double), stream),
               "memset");
    adj_G.assign(p.monitors.size(), nullptr);
    for (int q = 0; q < nmon; q++) {
      const Monitor &m = p.monitors[ids[q]];
      std::vector<double> h(grads[q], grads[q] + 2 * m.npts * m.freq.size());
      adj_G[ids[q]] = (double2 *)dupload(h);
    }
  }

  AdjCurlArgs<R> adj_args(Plan &p, int c) {
    const Plan::Curl &cp = p.curl[c];
    AdjCurlArgs<R> a{};
    a.lf = lam_f[c];
    a.lfu = lam_fu[c];
    a.xbar = xbar[c];
    a.dsig = cp.dsig;
    a.dsigu = cp.dsigu;
    for (int d = 0; d < 3; d++)
      a.shift[d] = p.shift[c][d];
    a.c = cp.flip ? -R(p.g.courant) : R(p.g.courant);
    a.box = full_box(p, c);
    a.dir = cdir(c);
    return a;
  }

  // gather description for the adjoint of source component srcc (E for B
  // curls, H for D curls)
  GatherArgs<R> gather_args(Plan &p, int srcc, int curl_type) {
    GatherArgs<R> ga{};
    int n = 0;
    for (int c = 0; c < NC; c++) {
      if (!p.have[c] || ctype(c) != curl_type) continue;
      const Plan::Curl &cp = p.curl[c];
      const int stp = curl_type == MFD_B ? 1 : -1;
      if (cp.g1 == srcc) ga.term[n++] = GatherTerm<R>{xbar[c], cp.d1, +1, stp};
      if (cp.g2 == srcc) ga.term[n++] = GatherTerm<R>{xbar[c], cp.d2, -1, stp};
    }
    ga.nterm = n;
    for (int q = 0; q < 3; q++) {
      ga.box.lo[q] = 0;
      ga.box.n[q] = p.ext[q];
      ga.N[q] = p.N[q];
    }
    return ga;
  }

  void adjoint_step(Plan &p, int64_t s, int64_t slot) override {
    join_dft();
    // 1. objective terms of the DFT samples taken after this step
    const int64_t tn = s + 1;
    for (size_t id = 0; id < p.monitors.size(); id++) {
      if (id >= adj_G.size() || !adj_G[id]) continue;
      const Monitor &m = p.monitors[id];
      if (tn % m.decimation != 0) continue;
      DMon &dm = mons[id];
      const int nf = (int)m.freq.size();
      double timeE = tn * p.dt;
      double time = (ctype(m.c) == MFD_H || ctype(m.c) == MFD_B) ? timeE - 0.5 * p.dt : timeE;
      // phases formed in the inject kernel's shared memory when they fit
      const bool inline_ph = size_t(nf) * sizeof(double2) <= 32768;
      if (!inline_ph) {
        dft_phase_kernel<<<(nf + 127) / 128, 128, 0, stream>>>(dm.freq, nf, time, m.scale.real(),
                                                                m.scale.imag(), dm.ph);
        nlaunch++;
      }
      InjectArgs<R> ia{};
      ia.lam = lam_f[m.c];
      ia.lamb = nullptr;
      if (ctype(m.c) == MFD_H) {
        int d = cdir(m.c);
        ia.hdir = d;
        ia.hshift = p.shift[m.c][d];
        ia.lamb = lam_f[comp(MFD_B, d)];
        if (!p.pml_dir[d]) ia.lam = ia.lamb;
      }
      for (int d = 0; d < 3; d++) {
        ia.w[d] = dm.w[d];
        ia.lo[d] = m.lo[d];
        ia.n[d] = m.hi[d] - m.lo[d] + 1;
      }
      ia.dV = m.dV;
      ia.include_weights = m.include_weights;
      ia.dim = p.g.dim;
      ia.ad0 = ia.ad1 = -1;
      if (m.centered)
        for (int d = 0; d < 3; d++)
          if (p.present[d] && p.shift[m.c][d] == 0) {
            if (ia.ad0 >= 0) ia.ad1 = d;
            else ia.ad0 = d;
          }
      ia.G = adj_G[id];
      ia.ph = inline_ph ? nullptr : dm.ph;
      ia.freq = dm.freq;
      ia.time = time;
      ia.sre = m.scale.real();
      ia.sim = m.scale.imag();
      ia.nf = nf;
      ia.npts = (long long)m.npts;
      adj_inject_kernel<R><<<(unsigned)((ia.npts + 255) / 256), 256, inline_ph ? size_t(nf) * sizeof(double2) : 0,
                             stream>>>(geo, ia);
      nlaunch++;
    }
    // 2-3. the 3-D band kernels when the forward runs them
    if (p.g.dim == 3 && fused_mask == MASK3) {
      adjoint_step3(p, slot);
      return;
    }
    // 2. reverse D/E half step
    for (int d = 0; d < 3; d++) {
      int c = comp(MFD_D, d);
      if (!p.have[c] || p.curl[c].g1 < 0) continue;
      AdjCurlArgs<R> a = adj_args(p, c);
      int ec = comp(MFD_E, d);
      a.le = lam_f[ec];
      a.lfw = lam_fw[ec];
      a.chi = chi[ec];
      a.isB = 0;
      a.gat = gather_args(p, ec, MFD_B);
      a.rec = nullptr;
      for (size_t q = 0; q < dcomps.size(); q++)
        if (dcomps[q] == ec && rec) {
          a.rec = rec + ((size_t)slot * dcomps.size() + q) * dnpts;
          a.grad = grad + q * dnpts;
          for (int e = 0; e < 3; e++) {
            a.dlo[e] = dbox.lo[e];
            a.dn[e] = dbox.n[e];
          }
        }
      dim3 grid, block;
      launch_dims(a.box, grid, block);
      adj_de_kernel<R><<<grid, block, 0, stream>>>(geo, tb, a);
      nlaunch++;
    }
    // 3. reverse B half step (H through f_w inside the slab, then the curl)
    std::vector<AdjCurlArgs<R>> bargs;
    for (int d = 0; d < 3; d++) {
      int c = comp(MFD_B, d);
      if (!p.have[c] || p.curl[c].g1 < 0) continue;
      AdjCurlArgs<R> a = adj_args(p, c);
      int hc = comp(MFD_H, d);
      a.le = p.pml_dir[d] ? lam_f[hc] : nullptr;
      a.lfw = lam_fw[hc];
      a.isB = 1;
      a.gat = gather_args(p, hc, MFD_D);
      bargs.push_back(a);
    }
    if (bargs.size() == 2 && bargs[0].box.n[geo.slow] == 1 && bargs[1].box.n[geo.slow] == 1) {
      // both B components in one launch (2-D)
      // one block shape for both, from the wider box; the grid covers both
      const int wide = bargs[0].box.n[geo.fast] >= bargs[1].box.n[geo.fast] ? 0 : 1;
      dim3 grid, block;
      launch_dims(bargs[wide].box, grid, block);
      for (const AdjCurlArgs<R> &a : bargs) {
        grid.x = std::max(grid.x, unsigned((a.box.n[geo.fast] + block.x - 1) / block.x));
        grid.y = std::max(grid.y, unsigned((a.box.n[geo.mid] + block.y - 1) / block.y));
      }
      grid.z = 2;
      adj_bh2_kernel<R><<<grid, block, 0, stream>>>(geo, tb, bargs[0], bargs[1]);
      nlaunch++;
    }
    else
      for (const AdjCurlArgs<R> &a : bargs) {
        dim3 grid, block;
        launch_dims(a.box, grid, block);
        adj_bh_kernel<R><<<grid, block, 0, stream>>>(geo, tb, a);
        nlaunch++;
      }
  }

  // reversed step on the 3-D bands: D/E (E part and D curl of all three
  // components per point), then B/H
  void adjoint_step3(Plan &p, int64_t slot) {
    Adj3Args<R> a{};
    a.g = fused_args(p, true);
    for (int d = 0; d < 3; d++) {
      a.lE[d] = lam_f[comp(MFD_E, d)];
      a.lfwE[d] = lam_fw[comp(MFD_E, d)];
      a.lD[d] = lam_f[comp(MFD_D, d)];
      a.lfuD[d] = lam_fu[comp(MFD_D, d)];
      a.xbD[d] = xbar[comp(MFD_D, d)];
      a.lH[d] = lam_f[comp(MFD_H, d)];
      a.lfwH[d] = lam_fw[comp(MFD_H, d)];
      a.lB[d] = lam_f[comp(MFD_B, d)];
      a.lfuB[d] = lam_fu[comp(MFD_B, d)];
      a.xbB[d] = xbar[comp(MFD_B, d)];
      a.chi[d] = chi[comp(MFD_E, d)];
      a.rec[d] = nullptr;
      a.grad[d] = nullptr;
      a.dlo[d] = dbox.lo[d];
      a.dn[d] = dbox.n[d];
    }
    a.c = R(p.g.courant);
    for (size_t q = 0; q < dcomps.size(); q++)
      if (rec && ctype(dcomps[q]) == MFD_E) {
        const int d = cdir(dcomps[q]);
        a.rec[d] = rec + ((size_t)slot * dcomps.size() + q) * dnpts;
        a.grad[d] = grad + q * dnpts;
      }
    const bool zp = a.g.pml[2] != 0;
    auto launch = [&](auto kern_tag, const Band &b, int kind, cudaStream_t st) {
      dim3 g, blk;
      band_shape(b, g, blk);
      if (g.x == 0) return;
      constexpr int which = decltype(kern_tag)::value;
      // kind: 0 rows, 1/2 full-row x/y faces, 3 xy edges, 4/5 z-interior x/y
      // faces, 6/7 their z edges
      const bool fx = kind == 1 || kind == 3 || kind == 4 || kind == 6;
      const bool fy = kind == 2 || kind == 3 || kind == 5 || kind == 7;
      const bool fz = zp && kind != 4 && kind != 5;
#define MFD_ADJ3(FX, FY, FZ)                                                                     \
  do {                                                                                             \
    if (which == 0) adj3_de_band_kernel<R, FX, FY, FZ><<<g, blk, 0, st>>>(a, b);                   \
    else adj3_bh_band_kernel<R, FX, FY, FZ><<<g, blk, 0, st>>>(a, b);                              \
  } while (0)
      if (fx && fy) {
        if (fz) MFD_ADJ3(true, true, true);
        else MFD_ADJ3(true, true, false);
      }
      else if (fx) {
        if (fz) MFD_ADJ3(true, false, true);
        else MFD_ADJ3(true, false, false);
      }
      else if (fy) {
        if (fz) MFD_ADJ3(false, true, true);
        else MFD_ADJ3(false, true, false);
      }
      else {
        if (fz) MFD_ADJ3(false, false, true);
        else MFD_ADJ3(false, false, false);
      }
#undef MFD_ADJ3
      nlaunch++;
    };
    over_bands3(p, [&](const Band &b, int kind, cudaStream_t st) {
      launch(std::integral_constant<int, 0>{}, b, kind, st);
    });
    over_bands3(p, [&](const Band &b, int kind, cudaStream_t st) {
      launch(std::integral_constant<int, 1>{}, b, kind, st);
    });
  }

  void adjoint_end(Plan &p, double *out) override {
    join_dft();
    (void)p;
    size_t n = dcomps.size() * dnpts;
    cuda_check(cudaMemcpyAsync(out, grad, n * sizeof(double), cudaMemcpyDeviceToHost, stream), "grad");
    cuda_check(cudaStreamSynchronize(stream), "grad sync");
    cuda_check(cudaGetLastError(), "adjoint");
  }

  void get_field_im(Plan &p, int c, double *out) override {
    join_dft();
    if (!cplx) {
      std::fill(out, out + p.ndense, 0.0);
      return;
    }
    swap_parts();
    try {
      get_field(p, c, out);
    } catch (...) {
      swap_parts();
      throw;
    }
    swap_parts();
  }

  void get_field(Plan &p, int c, double *out) override {
    join_dft();
    std::vector<R> h(p.nstore), hb;
    cuda_check(cudaMemcpyAsync(h.data(), f[c], p.nstore * sizeof(R), cudaMemcpyDeviceToHost, stream),
               "download");
    int t = ctype(c), d = cdir(c);
    bool sepH = t == MFD_H;
    if (sepH) {
      hb.resize(p.nstore);
      cuda_check(cudaMemcpyAsync(hb.data(), f[comp(MFD_B, d)], p.nstore * sizeof(R),
                                 cudaMemcpyDeviceToHost, stream),
                 "download");
    }
    cuda_check(cudaStreamSynchronize(stream), "download sync");
    for (int64_t di = 0; di < p.ndense; di++) {
      int k[3];
      p.dense_coords(di, k);
      int64_t i = k[0] * p.stride[0] + k[1] * p.stride[1] + k[2] * p.stride[2];
      if (sepH && !(p.pml_dir[d] && p.in_slab(d, p.shift[c][d] + 2 * k[d]))) out[di] = double(hb[i]);
      else out[di] = double(h[i]);
    }
  }

  void get_dft(Plan &p, int id, double *out) override {
    join_dft();
    dft_flush(p, id);
    const Monitor &m = p.monitors[id];
    size_t n = m.npts * m.freq.size();
    cuda_check(cudaMemcpyAsync(out, mons[id].acc, n * sizeof(double2), cudaMemcpyDeviceToHost, stream),
               "download dft");
    cuda_check(cudaStreamSynchronize(stream), "download sync");
    check_tc();
  }

  // Version of each monitor's sums, bumped by every change (a sample, set_dft,
  // scale_dft).  flux() returns its previous result for the same monitor
  // pairs while their versions are unchanged: the spectrum is a function of
  // the sums alone, so a caller reading the flux after every step (with a
  // decimated monitor) costs no device work or synchronisation on the steps
  // that add no sample.
  std::vector<unsigned long long> mon_ver;
  struct FluxMemo {
    std::vector<int> e, h;
    std::vector<unsigned long long> v;
    std::vector<double> out;
  };
  std::vector<FluxMemo> flux_memo;
  unsigned long long &ver(int id) {
    if ((size_t)id >= mon_ver.size()) mon_ver.resize(id + 1, 0);
    return mon_ver[id];
  }
  void bump(int id) { ver(id)++; }

  void flux(Plan &p, int npairs, const int *idE, const int *idH, double *out) override {
    join_dft();
    FluxMemo key;
    key.e.assign(idE, idE + npairs);
    key.h.assign(idH, idH + npairs);
    for (int q = 0; q < npairs; q++) {
      key.v.push_back(ver(idE[q]));
      key.v.push_back(ver(idH[q]));
    }
    for (const FluxMemo &m : flux_memo)
      if (m.e == key.e && m.h == key.h && m.v == key.v) {
        std::copy(m.out.begin(), m.out.end(), out);
        return;
      }
    for (int q = 0; q < npairs; q++) {
      dft_flush(p, idE[q]);
      dft_flush(p, idH[q]);
    }
    size_t nf = p.monitors[idE[0]].freq.size();
    const int maxparts = 512;
    if (flux_cap < nf) {
      d_flux = dalloc<double>(nf);
      d_flux_part = dalloc<double>((size_t)maxparts * nf);
      flux_cap = nf;
    }
    double *d_out = d_flux;
    for (int q = 0; q < npairs; q++) {
      long long np = (long long)p.monitors[idE[q]].npts;
      int gy = (int)std::min<long long>(std::max<long long>((np + 1023) / 1024, 1), maxparts);
      flux_partial_kernel<<<dim3((unsigned)((nf + 31) / 32), (unsigned)gy), dim3(32, 8), 0, stream>>>(
          mons[idE[q]].acc, mons[idH[q]].acc, np, (int)nf, d_flux_part);
      flux_final_kernel<<<(unsigned)((nf + 31) / 32), dim3(32, 8), 0, stream>>>(d_flux_part, gy, (int)nf, d_out,
                                                                               q > 0);
      nlaunch += 2;
    }
    cuda_check(cudaMemcpyAsync(out, d_out, nf * sizeof(double), cudaMemcpyDeviceToHost, stream),
               "download flux");
    cuda_check(cudaStreamSynchronize(stream), "flux sync");
    check_tc();
    key.out.assign(out, out + nf);
    if (flux_memo.size() >= 8) flux_memo.erase(flux_memo.begin());
    flux_memo.push_back(std::move(key));
  }

  void set_dft(Plan &p, int id, const double *in) override {
    join_dft();
    dft_flush(p, id);
    bump(id);
    const Monitor &m = p.monitors[id];
    cuda_check(cudaMemcpyAsync(mons[id].acc, in, m.npts * m.freq.size() * sizeof(double2), cudaMemcpyHostToDevice,
                               stream),
               "upload dft");
    cuda_check(cudaStreamSynchronize(stream), "upload dft sync");
    check_tc();
  }

  void scale_dft(Plan &p, int id, std::complex<double> sc) override {
    join_dft();
    dft_flush(p, id);
    bump(id);
    const Monitor &m = p.monitors[id];
    scale_device(mons[id].acc, (long long)(m.npts * m.freq.size()), sc.real(), sc.imag(), stream, nlaunch);
    cuda_check(cudaStreamSynchronize(stream), "scale sync");
    check_tc();
  }

  void farfield(Plan &p, const N2FSpec &s, const std::vector<N2FSheet> &sheets, int64_t nx, const double *x,
                double *out) override {
    join_dft();
    std::vector<N2FDevSheet> dev;
    for (const N2FSheet &sh : sheets) {
      dft_flush(p, sh.id);
      const Monitor &m = p.monitors[sh.id];
      N2FDevSheet d{};
      d.dft = mons[sh.id].acc;
      for (int q = 0; q < 3; q++) {
        d.n[q] = m.hi[q] - m.lo[q] + 1;
        d.is_half[q] = sh.is_half[q];
        d.rshift[q] = sh.rshift[q];
      }
      d.c0 = sh.c0;
      dev.push_back(d);
    }
    const std::vector<double> &fr = p.monitors[sheets[0].id].freq;
    farfield_device(s, dev, (int)fr.size(), fr.data(), nx, x, out, stream, nlaunch);
    check_tc();
  }
};

} // namespace cuda_impl
} // namespace mfd
