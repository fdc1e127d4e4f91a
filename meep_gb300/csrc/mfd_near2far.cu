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

#include "greens.hpp"
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
};

void check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw Error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

__global__ void __launch_bounds__(32 * N2F_WARPS)
    n2f_partial_kernel(const N2FParams P, const N2FDevSheet *__restrict__ sheets, const double *__restrict__ freq,
                       const double *__restrict__ xfar, double *__restrict__ part) {
  using namespace mgb_green;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long t = (long long)blockIdx.x * N2F_WARPS + warp;
  if (t >= P.npairs) return;
  const long long ix = t / P.nf;
  const int f = (int)(t - ix * P.nf);
  const double x[3] = {xfar[3 * ix], xfar[3 * ix + 1], xfar[3 * ix + 2]};
  const double fr = freq[f];
  const long long lo = (long long)blockIdx.y * P.seglen;
  const long long hi = min(lo + P.seglen, P.nsrc);
  const bool images = P.pn[0] > 0 || P.pn[1] > 0;
  double acc[12];
#pragma unroll
  for (int j = 0; j < 12; j++) acc[j] = 0.0;
  for (int m = 0; m < P.nsheet; m++) {
    const N2FDevSheet &S = sheets[m];
    const long long a = max(lo, S.start), b = min(hi, S.start + S.np);
    if (a >= b) continue;
    const int n1 = S.n[1], n2 = S.n[2], c0 = S.c0;
    const double2 *__restrict__ dft = S.dft;
    for (long long q = a + lane; q < b; q += 32) {
      const long long j = q - S.start;
      const long long r = j / n2;
      const int k2 = (int)(j - r * n2);
      const int k0 = (int)(r / n1);
      const int k1 = (int)(r - (long long)k0 * n1);
      // IVEC_LOOP_LOC, then the image shift
      double x0[3];
      x0[0] = __dadd_rn(__dmul_rn(S.is_half[0] + k0, P.inva), S.rshift[0]);
      x0[1] = __dadd_rn(__dmul_rn(S.is_half[1] + k1, P.inva), S.rshift[1]);
      x0[2] = __dadd_rn(__dmul_rn(S.is_half[2] + k2, P.inva), S.rshift[2]);
      if (P.dim == 2) x0[2] = 0.0;
      const double2 J = dft[j * P.nf + f];
      const cplx f0 = {J.x, J.y};
      cplx EH[6];
      if (!images) {
        if (P.dim == 2) green2d(EH, x, fr, P.eps, P.mu, x0, c0, f0);
        else green3d(EH, x, fr, P.eps, P.mu, x0, c0, f0);
#pragma unroll
        for (int c = 0; c < 6; c++) {
          acc[2 * c] += EH[c].re;
          acc[2 * c + 1] += EH[c].im;
        }
        continue;
      }
      double xs[3] = {x0[0], x0[1], x0[2]};
      for (int i0 = -P.pn[0]; i0 <= P.pn[0]; ++i0) {
        if (P.pdir[0] >= 0) xs[P.pdir[0]] = __dadd_rn(x0[P.pdir[0]], __dmul_rn(i0, P.period[0]));
        const double phase0 = i0 * P.pk[0];
        for (int i1 = -P.pn[1]; i1 <= P.pn[1]; ++i1) {
          if (P.pdir[1] >= 0) xs[P.pdir[1]] = __dadd_rn(x0[P.pdir[1]], __dmul_rn(i1, P.period[1]));
          const double phase = __dadd_rn(phase0, __dmul_rn(i1, P.pk[1]));
          const cplx cph = {cos(phase), sin(phase)};
          if (P.dim == 2) green2d(EH, x, fr, P.eps, P.mu, xs, c0, f0);
          else green3d(EH, x, fr, P.eps, P.mu, xs, c0, f0);
#pragma unroll
          for (int c = 0; c < 6; c++) {
            const cplx v = cmul(EH[c], cph);
            acc[2 * c] += v.re;
            acc[2 * c + 1] += v.im;
          }
        }
      }
    }
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

__global__ void green_kernel(int dim, int c0, double freq, double eps, double mu, double f0re, double f0im, long long n,
                             const double *__restrict__ x, const double *__restrict__ x0, double *__restrict__ out) {
  using namespace mgb_green;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double xa[3] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
  const double xb[3] = {x0[3 * i], x0[3 * i + 1], x0[3 * i + 2]};
  cplx EH[6];
  if (dim == 2) green2d(EH, xa, freq, eps, mu, xb, c0, cplx{f0re, f0im});
  else green3d(EH, xa, freq, eps, mu, xb, c0, cplx{f0re, f0im});
  for (int c = 0; c < 6; c++) {
    out[12 * i + 2 * c] = EH[c].re;
    out[12 * i + 2 * c + 1] = EH[c].im;
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
  n2f_partial_kernel<<<dim3((unsigned)bx, (unsigned)nseg), 32 * N2F_WARPS, 0, stream>>>(P, dsh, dfreq, dx, dpart);
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
  green_kernel<<<(unsigned)((n + 127) / 128), 128>>>(dim, c0, freq, eps, mu, f0re, f0im, (long long)n, dx, dx0, dout);
  check(cudaGetLastError(), "green_kernel launch");
  check(cudaMemcpy(out, dout, 12 * n * sizeof(double), cudaMemcpyDeviceToHost), "download Green's functions");
}

} // namespace mfd
