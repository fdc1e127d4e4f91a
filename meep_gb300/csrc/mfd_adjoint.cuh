// Reverse-time adjoint of the leapfrog step (exact discrete adjoint).
//
// One forward step is a sequence of linear updates with coefficients that do
// not depend on the fields: the curl updates of step_curl (four branches by
// PML direction, src/step_generic.cpp:94-248), H = B through f_w in the PML
// (src/step_generic.cpp:692-698) and E = chi1inv D (+ f_w inside the PML,
// src/step_generic.cpp:689-695, 773-776).  The adjoint applies the transposes
// in reverse order to adjoint fields lambda of the same shape; the only
// forward data it needs is D at the design points (for dJ/dchi1inv), which the
// forward pass records.  Objective terms enter as adjoint sources from
// dJ/dDFT: a DFT sum F = sum_n ph(n) v(n) gives dJ/dv(n) = Re(conj(G) ph(n)).
//
// Transposes used below (c = signed Courant factor, X = curl input):
//   plain            f' = f - cX                 : lf = lf',        Xb = -c lf'
//   u-PML            u' = u - cX, f' = su(kf+u'-u): lf = su k lf',  lu = lu',
//                                                   Xb = -c (lu' + su lf')
//   PML              f' = (ks f - cX) s          : lf = ks s lf',   Xb = -c s lf'
//   both             u' = (ks u - cX) s, f' = su(kf+u'-u):
//                    lt = lu' + su lf', lf = su k lf', lu = ks s lt - su lf',
//                    Xb = -c s lt
//   (k = kap_u - sig_u, su = siginv_u, ks = kap - sig, s = siginv)
// then Xb is gathered into the adjoint of the curl's source arrays.
#pragma once

namespace mfd {
namespace cuda_impl {

// Gather the curl adjoints Xb of up to two curl components into the adjoint
// of one source array (E for B curls; H or B for D curls).  For a curl term
// +G[i+s] - G[i] the adjoint of G receives +Xb at i+s and -Xb at i.
template <typename R> struct GatherTerm {
  const R *xb;   // Xb of the curl component (0 outside its updated points)
  int dir;       // direction of the stride s
  int sign;      // +1: term G[i+s] - G[i] (s along dir, +1 or -1 point); -1: G[i] - G[i+s]
  int step;      // +1 or -1: s = step * stride(dir)
};

template <typename R> struct GatherArgs {
  R *target;      // lambda array (B, or E)
  R *target_h;    // for D curls: lambda of H inside the H slab along hdir (null otherwise)
  int hdir;
  int nterm;
  GatherTerm<R> term[4];
  Box box;        // full point range of the source component
  int N[3];
};

// sum of the gathered curl adjoints at point j (k: its indices)
template <typename R> __device__ __forceinline__ R gather_at(const Geo &g, const GatherArgs<R> &a, const int k[3],
                                                             long long j) {
  R acc = R(0);
#pragma unroll
  for (int t = 0; t < 4; t++) {
    if (t >= a.nterm) break;
    const GatherTerm<R> &T = a.term[t];
    // term sign * (G[i+s] - G[i]): at point j the adjoint gets +Xb[j-s] - Xb[j]
    const int kn = k[T.dir] - T.step;
    R v = -T.xb[j];
    if (kn >= 0 && kn <= a.N[T.dir]) v += T.xb[j - T.step * g.stride[T.dir]];
    acc += T.sign > 0 ? v : -v;
  }
  return acc;
}

template <typename R> struct AdjCurlArgs {
  R *lf, *lfu, *xbar;
  int dsig, dsigu;
  int shift[3];
  R c; // signed Courant factor of the forward curl
  Box box;
  // E/H part
  int dir;
  R *le, *lfw;        // lambda of E (D curl) or H (B curl), and of its f_w
  const R *chi;       // E: chi1inv (D curl only)
  int isB;            // 1: B component (H part), 0: D component (E part)
  // gradient (D curl only): design box of this component
  const R *rec;       // recorded D at the design points for this step, or null
  double *grad;       // dJ/dchi1inv accumulator
  int dlo[3], dn[3];
  // curl adjoints of the other half step, gathered into the E (or H/B)
  // adjoint at this point before it is used
  GatherArgs<R> gat;
};

template <typename R>
__device__ __forceinline__ void adj_curl_core(const Geo &g, const Tables<R> &tb, const AdjCurlArgs<R> &a,
                                              const int k[3], long long i, R lam) {
  const bool sg = a.dsig >= 0 && slab(g, a.dsig, a.shift[a.dsig] + 2 * k[a.dsig]);
  const bool su = a.dsigu >= 0 && slab(g, a.dsigu, a.shift[a.dsigu] + 2 * k[a.dsigu]);
  R lf, xb;
  if (!sg && !su) {
    lf = lam;
    xb = -a.c * lam;
  }
  else if (!sg && su) {
    const int pu = a.shift[a.dsigu] + 2 * k[a.dsigu];
    const R siu = tb.siginv[a.dsigu][pu], ku = tb.kap[a.dsigu][pu] - tb.sig[a.dsigu][pu];
    const R lt = a.lfu[i] + siu * lam;
    lf = siu * ku * lam;
    xb = -a.c * lt;
    // lambda of f_u unchanged
  }
  else if (sg && !su) {
    const int ps = a.shift[a.dsig] + 2 * k[a.dsig];
    const R si = tb.siginv[a.dsig][ps], ks = tb.kap[a.dsig][ps] - tb.sig[a.dsig][ps];
    lf = ks * si * lam;
    xb = -a.c * si * lam;
  }
  else {
    const int ps = a.shift[a.dsig] + 2 * k[a.dsig];
    const int pu = a.shift[a.dsigu] + 2 * k[a.dsigu];
    const R si = tb.siginv[a.dsig][ps], ks = tb.kap[a.dsig][ps] - tb.sig[a.dsig][ps];
    const R siu = tb.siginv[a.dsigu][pu], ku = tb.kap[a.dsigu][pu] - tb.sig[a.dsigu][pu];
    const R lt = a.lfu[i] + siu * lam;
    lf = siu * ku * lam;
    a.lfu[i] = ks * si * lt - siu * lam;
    xb = -a.c * si * lt;
  }
  a.lf[i] = lf;
  a.xbar[i] = xb;
}

// Reverse of the D/E half step for one D component (E part, then the D curl).
template <typename R>
__global__ void __launch_bounds__(256) adj_de_kernel(Geo g, Tables<R> tb, AdjCurlArgs<R> a) {
  int k[3];
  if (!box_point(g, a.box, k)) return;
  const long long i = lin(g, k);
  // lambda of E: objective terms already added, plus the curl adjoints of the
  // B half step that read E
  const R le = a.le[i] + gather_at(g, a.gat, k, i);
  R lam = a.lf[i];
  const int pw = a.shift[a.dir] + 2 * k[a.dir];
  R gsrc;
  if (slab(g, a.dir, pw)) {
    // E' = E + (k+s) fw' - (k-s) fw, fw' = chi D'
    const R kk = tb.kap[a.dir][pw], ss = tb.sig[a.dir][pw];
    const R lfw = a.lfw[i] + (kk + ss) * le;
    a.lfw[i] = -(kk - ss) * le;
    a.le[i] = le; // lambda of E_old
    lam += a.chi[i] * lfw;
    gsrc = lfw;
  }
  else {
    // E' = chi (D' - P - sources)
    lam += a.chi[i] * le;
    a.le[i] = R(0);
    gsrc = le;
  }
  if (a.rec) {
    const int q0 = k[0] - a.dlo[0], q1 = k[1] - a.dlo[1], q2 = k[2] - a.dlo[2];
    if (q0 >= 0 && q0 < a.dn[0] && q1 >= 0 && q1 < a.dn[1] && q2 >= 0 && q2 < a.dn[2]) {
      const long long qi = ((long long)q0 * a.dn[1] + q1) * a.dn[2] + q2;
      a.grad[qi] += double(gsrc) * double(a.rec[qi]);
    }
  }
  adj_curl_core(g, tb, a, k, i, lam);
}

// Reverse of the B half step for one B component (H part, then the B curl).
template <typename R>
__device__ __forceinline__ void adj_bh_point(const Geo &g, const Tables<R> &tb, const AdjCurlArgs<R> &a,
                                             const int k[3]) {
  const long long i = lin(g, k);
  // curl adjoints of the D half step that read H (inside the H slab) or B
  const R gsum = gather_at(g, a.gat, k, i);
  R lam = a.lf[i];
  const int pw = 2 * k[a.dir];
  if (a.le && slab(g, a.dir, pw)) {
    // H' = H + (k+s) B' - (k-s) fw, fw' = B'
    const R kk = tb.kap[a.dir][pw], ss = tb.sig[a.dir][pw];
    const R lh = a.le[i] + gsum;
    a.le[i] = lh;
    lam += (kk + ss) * lh + a.lfw[i];
    a.lfw[i] = -(kk - ss) * lh;
  }
  else
    lam += gsum;
  adj_curl_core(g, tb, a, k, i, lam);
}

template <typename R>
__global__ void __launch_bounds__(256) adj_bh_kernel(Geo g, Tables<R> tb, AdjCurlArgs<R> a) {
  int k[3];
  if (!box_point(g, a.box, k)) return;
  adj_bh_point(g, tb, a, k);
}

// Two B components of a grid whose slow direction is one point thick (2-D):
// blockIdx.z picks the component.  The reversed B updates of different
// components touch disjoint arrays, so one launch does both.
template <typename R>
__global__ void __launch_bounds__(256) adj_bh2_kernel(Geo g, Tables<R> tb, AdjCurlArgs<R> a0, AdjCurlArgs<R> a1) {
  const AdjCurlArgs<R> &a = blockIdx.z ? a1 : a0;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= a.box.n[g.fast] || m >= a.box.n[g.mid] || a.box.n[g.slow] < 1) return;
  int k[3];
  k[g.fast] = a.box.lo[g.fast] + x;
  k[g.mid] = a.box.lo[g.mid] + m;
  k[g.slow] = a.box.lo[g.slow];
  adj_bh_point(g, tb, a, k);
}

template <typename R> __global__ void __launch_bounds__(256) adj_gather_kernel(Geo g, GatherArgs<R> a) {
  int k[3];
  if (!box_point(g, a.box, k)) return;
  const long long j = lin(g, k);
  R acc = R(0);
#pragma unroll
  for (int t = 0; t < 4; t++) {
    if (t >= a.nterm) break;
    const GatherTerm<R> &T = a.term[t];
    // term sign * (G[i+s] - G[i]): at point j the adjoint gets +Xb[j-s] - Xb[j]
    const int kn = k[T.dir] - T.step;
    R v = -T.xb[j];
    if (kn >= 0 && kn <= a.N[T.dir]) v += T.xb[j - T.step * g.stride[T.dir]];
    acc += T.sign > 0 ? v : -v;
  }
  R *tgt = a.target;
  if (a.target_h && slab(g, a.hdir, 2 * k[a.hdir])) tgt = a.target_h;
  tgt[j] += acc;
}

// Adjoint sources of one monitor at one sampled step: value v(p) of the
// monitor (weighted, centred) gets dJ/dv = Re(conj(G[p][w]) ph[w]); spread to
// the averaged component points.
template <typename R> struct InjectArgs {
  R *lam, *lamb; // component lambda; for H components lambda of B outside the H slab
  int hdir, hshift;
  const double *w[3];
  double dV;
  int include_weights, dim;
  int lo[3], n[3];
  int ad0, ad1;
  const double2 *G;  // [npts][nf]
  const double2 *ph; // [nf] phases of this sample, or null: formed per block
  const double *freq; // with ph null: scale * exp(2 pi i f time) per block
  double time, sre, sim;
  int nf;
  long long npts;
};

template <typename R> __device__ __forceinline__ void inj_add(const Geo &g, const InjectArgs<R> &a, const int k[3], double v) {
  const long long i = lin(g, k);
  R *t = a.lam;
  if (a.lamb && !slab(g, a.hdir, a.hshift + 2 * k[a.hdir])) t = a.lamb;
  atomicAdd(t + i, R(v));
}

template <typename R> __global__ void adj_inject_kernel(Geo g, InjectArgs<R> a) {
  extern __shared__ double2 sph[];
  const double2 *phase = a.ph;
  if (!phase) {
    // the sample's phases, as dft_phase_kernel forms them
    for (int w = threadIdx.x; w < a.nf; w += blockDim.x) {
      double s, c;
      sincos(2 * kPi * a.freq[w] * a.time, &s, &c);
      sph[w] = make_double2(c * a.sre - s * a.sim, c * a.sim + s * a.sre);
    }
    __syncthreads();
    phase = sph;
  }
  long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= a.npts) return;
  double s = 0;
  for (int w = 0; w < a.nf; w++) {
    const double2 G = a.G[p * a.nf + w], ph = phase[w];
    s += G.x * ph.x + G.y * ph.y;
  }
  if (s == 0) return;
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
  }
  if (a.ad1 >= 0) {
    const double v = s * wgt * 0.25;
    int k1[3] = {k[0], k[1], k[2]}, k2[3] = {k[0], k[1], k[2]}, k3[3] = {k[0], k[1], k[2]};
    k1[a.ad0]++;
    k2[a.ad1]++;
    k3[a.ad0]++;
    k3[a.ad1]++;
    inj_add(g, a, k, v);
    inj_add(g, a, k1, v);
    inj_add(g, a, k2, v);
    inj_add(g, a, k3, v);
  }
  else if (a.ad0 >= 0) {
    const double v = s * wgt * 0.5;
    int k1[3] = {k[0], k[1], k[2]};
    k1[a.ad0]++;
    inj_add(g, a, k, v);
    inj_add(g, a, k1, v);
  }
  else
    inj_add(g, a, k, s * wgt);
}

// design-box copy of one component (forward recording)
template <typename R> __global__ void box_copy_kernel(Geo g, const R *src, R *dst, Box b) {
  int k[3];
  if (!box_point(g, b, k)) return;
  const long long qi = ((long long)(k[0] - b.lo[0]) * b.n[1] + (k[1] - b.lo[1])) * b.n[2] + (k[2] - b.lo[2]);
  dst[qi] = src[lin(g, k)];
}

} // namespace cuda_impl
} // namespace mfd
