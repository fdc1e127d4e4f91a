// Near-to-far transform on the GPU.
//
// The far field at x is a sum over every point of every equivalent current
// sheet (and its periodic images) of a Green's function times the point's DFT
// sum (dft_near2far::farfield_lowlevel, src/near2far.cpp:334-378).  Each
// Green's function is different (it depends on x - x0 and the frequency), so
// there is no operand reuse for the tensor cores: the work is FP64 arithmetic
// on the CUDA cores (sqrt, sin/cos or the Bessel functions, a few divisions),
// reading 16 bytes of DFT sum per evaluation from L2.
//
// Decomposition: one warp per (far point, frequency) pair, its lanes striding
// over a segment of the flattened source points; segments along grid.y give
// enough warps when there are few pairs.  Each warp reduces its 12 partial
// sums with a fixed shuffle tree and writes them per segment; a second kernel
// adds the segments in order, so results are reproducible run to run.
#include <algorithm>
#include <string>

#include "greens.hpp" // mgb_green::PI
#include "mfd_near2far.hpp"

namespace mfd {

namespace {

constexpr int N2F_WARPS = 8;

struct N2FParams {
  int dim, nsheet, nf;
  long long npairs, nsrc, seglen;
  double eps, mu, inva;
  int pdir[2], pn[2];
  double pk[2], period[2];
  double freq_f; // set per warp: the warp's frequency
};

void check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw Error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

/* Device forms of green3d / green2d (greens.hpp holds the reference-order
   host form).  The same formulas, rearranged for the FP64 pipe, which bounds
   this kernel: the per-frequency and per-medium factors (k, 1/k, Z, 1/Z,
   k n / (4 pi) / eps, ...) are computed once per sheet, the current
   direction is a template parameter (p = e_d, so the products with its zero
   components vanish), 1/r comes from rsqrt, 1/(kr) = (1/r)(1/k),
   exp(i (kr + pi/2)) = i exp(i kr), a lattice image's Bloch phase multiplies
   the source amplitude instead of the six results, and in 2-D the Hankel
   function of order 2 comes from orders 0 and 1 (H2 = (2 / kr) H1 - H0)
   instead of a third pair of Bessel calls.  Each result differs from the
   reference-order evaluation by a few units in the last place. */
struct GConst {
  double k, inv_k; // wavenumber in the medium and its inverse
  double amp;      // 3-D: k n / (4 pi) / (eps or mu)
  double Z, invZ;  // sqrt(mu / eps) and its inverse
  double h0;       // 2-D: -omega mu / 4 (electric), -omega eps / 4 (magnetic)
  double a;        // 2-D: Z / 4 (electric), 1 / (4 Z) (magnetic)
  double b;        // 2-D: omega mu / 8 (electric), omega eps / 8 (magnetic)
  double qk;       // 2-D: k / 4
};

__device__ __forceinline__ GConst make_gconst(int dim, bool electric, double freq, double eps, double mu) {
  using mgb_green::PI;
  GConst g;
  const double n = sqrt(eps * mu);
  const double omega = 2 * PI * freq;
  g.k = omega * n;
  g.inv_k = 1.0 / g.k;
  g.Z = sqrt(mu / eps);
  g.invZ = 1.0 / g.Z;
  g.amp = g.k * n / (4 * PI) / (electric ? eps : mu);
  g.h0 = -0.25 * omega * (electric ? mu : eps);
  g.a = electric ? 0.25 * g.Z : 0.25 * g.invZ;
  g.b = 0.125 * omega * (electric ? mu : eps);
  g.qk = 0.25 * g.k;
  (void)dim;
  return g;
}

// acc[2c], acc[2c+1] += fields of a current f0 along C0 (0..2 E, 3..5 H)
template <int C0>
__device__ __forceinline__ void green3d_acc(const GConst &g, const double x[3], const double x0[3], double fr,
                                            double fi, double acc[12]) {
  constexpr int d = C0 % 3;
  constexpr bool electric = C0 < 3;
  const double v0 = x[0] - x0[0], v1 = x[1] - x0[1], v2 = x[2] - x0[2];
  const double r2 = v0 * v0 + v1 * v1 + v2 * v2;
  const double inv_r = rsqrt(r2);
  const double r = r2 * inv_r;
  const double u[3] = {v0 * inv_r, v1 * inv_r, v2 * inv_r};
  const double kr = g.k * r;
  const double ikr = inv_r * g.inv_k; // 1 / (kr)
  const double q = ikr * ikr;
  double sn, cs;
  sincos(kr, &sn, &cs);
  // e = f0 * amp / r * exp(i (kr + pi / 2)) = f0 * (amp / r) * (-sin kr, cos kr)
  const double ar = g.amp * inv_r;
  const double pr = -ar * sn, pi_ = ar * cs;
  const double er = fr * pr - fi * pi_, ei = fr * pi_ + fi * pr;
  const double pd = u[d];
  // t1 = (1 - q, 1/kr); t2 = ((3q - 1) p.r, -3 p.r / kr); t3 = (1, 1/kr)
  const double t2r = (3.0 * q - 1.0) * pd, t2i = -3.0 * ikr * pd;
  const double et2r = er * t2r - ei * t2i, et2i = er * t2i + ei * t2r;
  const double t1r = 1.0 - q;
  double Ar[3], Ai[3];
#pragma unroll
  for (int j = 0; j < 3; j++) {
    Ar[j] = et2r * u[j];
    Ai[j] = et2i * u[j];
  }
  Ar[d] += er * t1r - ei * ikr;
  Ai[d] += er * ikr + ei * t1r;
  // e t3 and r x p with p = e_d: rxp = (u1 p2 - u2 p1, u2 p0 - u0 p2, u0 p1 - u1 p0)
  const double e3r = er - ei * ikr, e3i = er * ikr + ei;
  double rxp[3] = {0.0, 0.0, 0.0};
  if (d == 0) rxp[1] = u[2], rxp[2] = -u[1];
  if (d == 1) rxp[0] = -u[2], rxp[2] = u[0];
  if (d == 2) rxp[0] = u[1], rxp[1] = -u[0];
  const double s = electric ? g.invZ : -g.Z;
  const double br = e3r * s, bi = e3i * s;
  constexpr int oA = electric ? 0 : 6, oB = electric ? 6 : 0;
#pragma unroll
  for (int j = 0; j < 3; j++) {
    acc[oA + 2 * j] += Ar[j];
    acc[oA + 2 * j + 1] += Ai[j];
    if (j != d) {
      acc[oB + 2 * j] += br * rxp[j];
      acc[oB + 2 * j + 1] += bi * rxp[j];
    }
  }
}

template <int C0>
__device__ __forceinline__ void green2d_acc(const GConst &g, const double x[3], const double x0[3], double fr,
                                            double fi, double acc[12]) {
  constexpr int d = C0 % 3;
  constexpr bool electric = C0 < 3;
  const double v0 = x[0] - x0[0], v1 = x[1] - x0[1];
  const double r2 = v0 * v0 + v1 * v1;
  const double inv_r = rsqrt(r2);
  const double r = r2 * inv_r;
  const double u0 = v0 * inv_r, u1 = v1 * inv_r;
  const double kr = g.k * r;
  const double J0 = j0(kr), Y0 = y0(kr), J1 = j1(kr), Y1 = y1(kr);
  // H_n f0
  const double h0r = J0 * fr - Y0 * fi, h0i = J0 * fi + Y0 * fr;
  const double h1r = J1 * fr - Y1 * fi, h1i = J1 * fi + Y1 * fr;
  // i k / 4 H1
  const double kh1r = -g.qk * h1i, kh1i = g.qk * h1r;
  if (d == 2) {
    if (electric) {
      acc[4] += g.h0 * h0r;
      acc[5] += g.h0 * h0i;
      acc[6] += -u1 * kh1r;
      acc[7] += -u1 * kh1i;
      acc[8] += u0 * kh1r;
      acc[9] += u0 * kh1i;
    }
    else {
      acc[0] += u1 * kh1r;
      acc[1] += u1 * kh1i;
      acc[2] += -u0 * kh1r;
      acc[3] += -u0 * kh1i;
      acc[10] += g.h0 * h0r;
      acc[11] += g.h0 * h0i;
    }
    return;
  }
  // H0 - H2 = 2 H0 - (2 / kr) H1
  const double tk = 2.0 * inv_r * g.inv_k;
  const double dr = 2.0 * h0r - tk * h1r, di = 2.0 * h0i - tk * h1i;
  const double pd = d == 0 ? u0 : u1;
  const double rxp = d == 0 ? -u1 : u0;
  const double a = pd * inv_r * g.a, b = rxp * g.b;
  const int o = electric ? 0 : 6;
  acc[o + 0] += -(u0 * a) * h1r + (u1 * b) * dr;
  acc[o + 1] += -(u0 * a) * h1i + (u1 * b) * di;
  acc[o + 2] += -(u1 * a) * h1r - (u0 * b) * dr;
  acc[o + 3] += -(u1 * a) * h1i - (u0 * b) * di;
  const int oz = electric ? 10 : 4;
  const double sz = electric ? -rxp : rxp;
  acc[oz] += sz * kh1r;
  acc[oz + 1] += sz * kh1i;
}

template <int DIM, int C0>
__device__ __forceinline__ void green_acc(const GConst &g, const double x[3], const double x0[3], double fr, double fi,
                                          double acc[12]) {
  if (DIM == 2) green2d_acc<C0>(g, x, x0, fr, fi, acc);
  else green3d_acc<C0>(g, x, x0, fr, fi, acc);
}

// this lane's points q = a + lane, a + lane + 32, ... < b of one sheet
template <int DIM, int C0>
__device__ __forceinline__ void sheet_sum(const N2FParams &P, const N2FDevSheet &S, long long a, long long b, int lane,
                                          int f, const double x[3], double acc[12]) {
  const GConst g = make_gconst(DIM, C0 < 3, 0.0 + P.freq_f, P.eps, P.mu);
  const int n1 = S.n[1], n2 = S.n[2];
  const double2 *__restrict__ dft = S.dft;
  const bool images = P.pn[0] > 0 || P.pn[1] > 0;
  for (long long q = a + lane; q < b; q += 32) {
    const long long j = q - S.start;
    const long long rr = j / n2;
    const int k2 = (int)(j - rr * n2);
    const int k0 = (int)(rr / n1);
    const int k1 = (int)(rr - (long long)k0 * n1);
    // IVEC_LOOP_LOC, then the image shift
    double x0[3];
    x0[0] = __dadd_rn(__dmul_rn(S.is_half[0] + k0, P.inva), S.rshift[0]);
    x0[1] = __dadd_rn(__dmul_rn(S.is_half[1] + k1, P.inva), S.rshift[1]);
    x0[2] = DIM == 2 ? 0.0 : __dadd_rn(__dmul_rn(S.is_half[2] + k2, P.inva), S.rshift[2]);
    const double2 J = dft[j * P.nf + f];
    if (!images) {
      green_acc<DIM, C0>(g, x, x0, J.x, J.y, acc);
      continue;
    }
    double xs[3] = {x0[0], x0[1], x0[2]};
    for (int i0 = -P.pn[0]; i0 <= P.pn[0]; ++i0) {
      if (P.pdir[0] >= 0) xs[P.pdir[0]] = __dadd_rn(x0[P.pdir[0]], __dmul_rn(i0, P.period[0]));
      const double phase0 = i0 * P.pk[0];
      for (int i1 = -P.pn[1]; i1 <= P.pn[1]; ++i1) {
        if (P.pdir[1] >= 0) xs[P.pdir[1]] = __dadd_rn(x0[P.pdir[1]], __dmul_rn(i1, P.period[1]));
        double sn, cs;
        sincos(__dadd_rn(phase0, __dmul_rn(i1, P.pk[1])), &sn, &cs);
        // the image's Bloch phase on the source amplitude (linear in f0)
        green_acc<DIM, C0>(g, x, xs, J.x * cs - J.y * sn, J.x * sn + J.y * cs, acc);
      }
    }
  }
}

template <int DIM>
__device__ __forceinline__ void sheet_dispatch(const N2FParams &P, const N2FDevSheet &S, long long a, long long b,
                                               int lane, int f, const double x[3], double acc[12]) {
  switch (S.c0) {
    case 0: sheet_sum<DIM, 0>(P, S, a, b, lane, f, x, acc); break;
    case 1: sheet_sum<DIM, 1>(P, S, a, b, lane, f, x, acc); break;
    case 2: sheet_sum<DIM, 2>(P, S, a, b, lane, f, x, acc); break;
    case 3: sheet_sum<DIM, 3>(P, S, a, b, lane, f, x, acc); break;
    case 4: sheet_sum<DIM, 4>(P, S, a, b, lane, f, x, acc); break;
    default: sheet_sum<DIM, 5>(P, S, a, b, lane, f, x, acc); break;
  }
}

template <int DIM>
__global__ void __launch_bounds__(32 * N2F_WARPS)
    n2f_partial_kernel(N2FParams P, const N2FDevSheet *__restrict__ sheets, const double *__restrict__ freq,
                       const double *__restrict__ xfar, double *__restrict__ part) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long t = (long long)blockIdx.x * N2F_WARPS + warp;
  if (t >= P.npairs) return;
  const long long ix = t / P.nf;
  const int f = (int)(t - ix * P.nf);
  const double x[3] = {xfar[3 * ix], xfar[3 * ix + 1], DIM == 2 ? 0.0 : xfar[3 * ix + 2]};
  P.freq_f = freq[f];
  const long long lo = (long long)blockIdx.y * P.seglen;
  const long long hi = min(lo + P.seglen, P.nsrc);
  double acc[12];
#pragma unroll
  for (int j = 0; j < 12; j++) acc[j] = 0.0;
  for (int m = 0; m < P.nsheet; m++) {
    const N2FDevSheet &S = sheets[m];
    const long long a = max(lo, S.start), b = min(hi, S.start + S.np);
    if (a < b) sheet_dispatch<DIM>(P, S, a, b, lane, f, x, acc);
  }
#pragma unroll
  for (int j = 0; j < 12; j++) {
    double v = acc[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    acc[j] = v;
  }
  if (lane == 0) {
    double *dst = part + ((long long)blockIdx.y * P.npairs + t) * 12;
#pragma unroll
    for (int j = 0; j < 12; j++) dst[j] = acc[j];
  }
}

// out[i] = sum over segments g (in order) of part[g * n + i]
__global__ void n2f_reduce_kernel(const double *__restrict__ part, int nseg, long long n, double *__restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int g = 0; g < nseg; g++) s += part[(long long)g * n + i];
  out[i] = s;
}

__global__ void scale_kernel(double2 *v, long long n, double sre, double sim) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  // (ac - bd, ad + bc) rounded term by term, as the host's complex product
  const double2 a = v[i];
  v[i] = make_double2(__dsub_rn(__dmul_rn(a.x, sre), __dmul_rn(a.y, sim)),
                      __dadd_rn(__dmul_rn(a.x, sim), __dmul_rn(a.y, sre)));
}

template <int DIM, int C0>
__device__ __forceinline__ void green_one(const GConst &g, const double *xa, const double *xb, double f0re,
                                          double f0im, double *o) {
  double acc[12];
#pragma unroll
  for (int j = 0; j < 12; j++) acc[j] = 0.0;
  green_acc<DIM, C0>(g, xa, xb, f0re, f0im, acc);
#pragma unroll
  for (int j = 0; j < 12; j++) o[j] = acc[j];
}

// mfd_green: the device forms the far-field kernel uses, one pair per thread
template <int DIM>
__global__ void green_kernel(int c0, double freq, double eps, double mu, double f0re, double f0im, long long n,
                             const double *__restrict__ x, const double *__restrict__ x0, double *__restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double xa[3] = {x[3 * i], x[3 * i + 1], DIM == 2 ? 0.0 : x[3 * i + 2]};
  const double xb[3] = {x0[3 * i], x0[3 * i + 1], DIM == 2 ? 0.0 : x0[3 * i + 2]};
  const GConst g = make_gconst(DIM, c0 < 3, freq, eps, mu);
  double *o = out + 12 * i;
  switch (c0) {
    case 0: green_one<DIM, 0>(g, xa, xb, f0re, f0im, o); break;
    case 1: green_one<DIM, 1>(g, xa, xb, f0re, f0im, o); break;
    case 2: green_one<DIM, 2>(g, xa, xb, f0re, f0im, o); break;
    case 3: green_one<DIM, 3>(g, xa, xb, f0re, f0im, o); break;
    case 4: green_one<DIM, 4>(g, xa, xb, f0re, f0im, o); break;
    default: green_one<DIM, 5>(g, xa, xb, f0re, f0im, o); break;
  }
}

struct Buffers {
  std::vector<void *> ptrs;
  template <class T> T *alloc(size_t n) {
    void *p = nullptr;
    check(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)), "cudaMalloc");
    ptrs.push_back(p);
    return static_cast<T *>(p);
  }
  ~Buffers() {
    for (void *p : ptrs) cudaFree(p);
  }
};

} // namespace

void farfield_device(const N2FSpec &s, std::vector<N2FDevSheet> sheets, int nf, const double *freq, int64_t nx,
                     const double *x, double *out, cudaStream_t stream, long long &nlaunch) {
  long long nsrc = 0;
  for (N2FDevSheet &S : sheets) {
    S.start = nsrc;
    S.np = (long long)S.n[0] * S.n[1] * S.n[2];
    nsrc += S.np;
  }
  const long long npairs = (long long)nx * nf;
  if (npairs == 0) return;
  if (nsrc == 0) {
    std::fill(out, out + npairs * 12, 0.0);
    return;
  }
  int dev = 0, sms = 0;
  check(cudaGetDevice(&dev), "cudaGetDevice");
  check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
  // enough warps for every SM (32 resident per SM), each with at least 8
  // source points per lane
  const long long want_warps = (long long)sms * 32;
  long long nseg = std::max<long long>(1, (want_warps + npairs - 1) / npairs);
  nseg = std::min<long long>(nseg, std::max<long long>(1, nsrc / 256));
  nseg = std::min<long long>(nseg, 65535);
  const long long seglen = (nsrc + nseg - 1) / nseg;
  nseg = (nsrc + seglen - 1) / seglen;
  const long long bx = (npairs + N2F_WARPS - 1) / N2F_WARPS;
  if (bx > 0x7fffffffLL) throw Error("farfield: too many far points x frequencies for one call");

  N2FParams P{};
  P.dim = s.dim;
  P.nsheet = (int)sheets.size();
  P.nf = nf;
  P.npairs = npairs;
  P.nsrc = nsrc;
  P.seglen = seglen;
  P.eps = s.eps;
  P.mu = s.mu;
  P.inva = s.inva;
  for (int i = 0; i < 2; i++) {
    P.pdir[i] = s.pdir[i];
    P.pn[i] = s.pn[i];
    P.pk[i] = s.pk[i];
    P.period[i] = s.period[i];
  }
  Buffers b;
  N2FDevSheet *dsh = b.alloc<N2FDevSheet>(sheets.size());
  double *dfreq = b.alloc<double>(nf), *dx = b.alloc<double>(3 * nx);
  double *dpart = b.alloc<double>((size_t)nseg * npairs * 12), *dout = b.alloc<double>((size_t)npairs * 12);
  check(cudaMemcpyAsync(dsh, sheets.data(), sheets.size() * sizeof(N2FDevSheet), cudaMemcpyHostToDevice, stream),
        "upload sheets");
  check(cudaMemcpyAsync(dfreq, freq, nf * sizeof(double), cudaMemcpyHostToDevice, stream), "upload frequencies");
  check(cudaMemcpyAsync(dx, x, 3 * nx * sizeof(double), cudaMemcpyHostToDevice, stream), "upload far points");
  if (s.dim == 2)
    n2f_partial_kernel<2><<<dim3((unsigned)bx, (unsigned)nseg), 32 * N2F_WARPS, 0, stream>>>(P, dsh, dfreq, dx, dpart);
  else
    n2f_partial_kernel<3><<<dim3((unsigned)bx, (unsigned)nseg), 32 * N2F_WARPS, 0, stream>>>(P, dsh, dfreq, dx, dpart);
  check(cudaGetLastError(), "n2f_partial_kernel launch");
  const long long nout = npairs * 12;
  n2f_reduce_kernel<<<(unsigned)((nout + 255) / 256), 256, 0, stream>>>(dpart, (int)nseg, nout, dout);
  check(cudaGetLastError(), "n2f_reduce_kernel launch");
  nlaunch += 2;
  check(cudaMemcpyAsync(out, dout, nout * sizeof(double), cudaMemcpyDeviceToHost, stream), "download far fields");
  check(cudaStreamSynchronize(stream), "far-field sync");
}

void scale_device(double2 *v, long long n, double sre, double sim, cudaStream_t stream, long long &nlaunch) {
  if (n <= 0) return;
  scale_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(v, n, sre, sim);
  check(cudaGetLastError(), "scale_kernel launch");
  nlaunch++;
}

void green_eval(int dim, int c0, double freq, double eps, double mu, double f0re, double f0im, int64_t n,
                const double *x, const double *x0, double *out) {
  if (n <= 0) return;
  Buffers b;
  double *dx = b.alloc<double>(3 * n), *dx0 = b.alloc<double>(3 * n), *dout = b.alloc<double>(12 * n);
  check(cudaMemcpy(dx, x, 3 * n * sizeof(double), cudaMemcpyHostToDevice), "upload points");
  check(cudaMemcpy(dx0, x0, 3 * n * sizeof(double), cudaMemcpyHostToDevice), "upload source points");
  if (dim == 2)
    green_kernel<2><<<(unsigned)((n + 127) / 128), 128>>>(c0, freq, eps, mu, f0re, f0im, (long long)n, dx, dx0, dout);
  else
    green_kernel<3><<<(unsigned)((n + 127) / 128), 128>>>(c0, freq, eps, mu, f0re, f0im, (long long)n, dx, dx0, dout);
  check(cudaGetLastError(), "green_kernel launch");
  check(cudaMemcpy(out, dout, 12 * n * sizeof(double), cudaMemcpyDeviceToHost), "download Green's functions");
}

} // namespace mfd
