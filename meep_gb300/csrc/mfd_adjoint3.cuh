// Reverse-time adjoint of the 3-D step on the band decomposition of the
// forward kernels (mfd_k3d.cuh): one launch set per reversed half-step that
// handles all three components of a point, instead of one grid-wide launch per
// component (mfd_adjoint.cuh, which holds the derivation and the transposes).
// Per point the arithmetic is that of adj_de_kernel / adj_bh_kernel with the
// gather terms in the same order, so the gradient is the same to the bit.
//
// 3-D curl plan (Plan::curl): B_d -= c (E_{d+2}[i+s_{d+1}] - E_{d+2}[i] +
// E_{d+1}[i] - E_{d+1}[i+s_{d+2}]); D_d likewise from H with backward
// neighbours.  The adjoint of the curl input (xbar of each D/B component) is
// pulled into lambda of E (H) at every point by the next reversed half-step:
//   E_x <- +xbar(B_y) along z, -xbar(B_z) along y   (forward neighbours)
//   E_y <- -xbar(B_x) along z, +xbar(B_z) along x
//   E_z <- +xbar(B_x) along y, -xbar(B_y) along x
//   H_x <- +xbar(D_y) along z, -xbar(D_z) along y   (backward neighbours)
//   H_y <- -xbar(D_x) along z, +xbar(D_z) along x
//   H_z <- +xbar(D_x) along y, -xbar(D_y) along x
#pragma once

namespace mfd {
namespace cuda_impl {

template <typename R> struct Adj3Args {
  FusedArgs<R> g; // geometry and PML tables (N, T, pml, s, sig, kap, siginv)
  R *lE[3], *lfwE[3], *lD[3], *lfuD[3], *xbD[3];
  R *lH[3], *lfwH[3], *lB[3], *lfuB[3], *xbB[3];
  const R *chi[3];
  R c; // Courant factor (no flipped curls in 3-D)
  // design gradient per E component (null: not a design component)
  const R *rec[3];
  double *grad[3];
  int dlo[3], dn[3];
};

// one gather term: sign * (-xb[j] + xb[j -/+ s]) with the neighbour in range
template <typename R, int STEP>
__device__ __forceinline__ R gterm(const R *xb, const FusedArgs<R> &g, const int k[3], int i, int dir) {
  R v = -xb[i];
  const int kn = k[dir] - STEP;
  if (kn >= 0 && kn <= g.N[dir]) v += xb[i - STEP * g.s[dir]];
  return v;
}

// adjoint of step_curl's branches for one component (adj_curl_core), with
// lambda of f_u already loaded (lfuv): returns lambda of f, xbar and the new
// lambda of f_u (written only when both slabs apply)
template <typename R> struct AdjCurl3 {
  R lf, xb, lfu;
};
template <typename R>
__device__ __forceinline__ AdjCurl3<R> adj3_curl(const FusedArgs<R> &g, R c, bool sg, bool su, int ds, int ps,
                                                 int du, int pu, R lfuv, R lam) {
  AdjCurl3<R> o;
  o.lfu = lfuv;
  if (!sg && !su) {
    o.lf = lam;
    o.xb = -c * lam;
  }
  else if (!sg && su) {
    const R siu = g.siginv[du][pu], ku = g.kap[du][pu] - g.sig[du][pu];
    const R lt = lfuv + siu * lam;
    o.lf = siu * ku * lam;
    o.xb = -c * lt;
  }
  else if (sg && !su) {
    const R si = g.siginv[ds][ps], ks = g.kap[ds][ps] - g.sig[ds][ps];
    o.lf = ks * si * lam;
    o.xb = -c * si * lam;
  }
  else {
    const R si = g.siginv[ds][ps], ks = g.kap[ds][ps] - g.sig[ds][ps];
    const R siu = g.siginv[du][pu], ku = g.kap[du][pu] - g.sig[du][pu];
    const R lt = lfuv + siu * lam;
    o.lf = siu * ku * lam;
    o.lfu = ks * si * lt - siu * lam;
    o.xb = -c * si * lt;
  }
  return o;
}

// gathered curl adjoints of the other half-step into component d (terms of
// the forward curl plan, in its order)
template <typename R, int STEP>
__device__ __forceinline__ R gather3(const FusedArgs<R> &g, R *const *xb, int d, const int k[3], int i) {
  R acc = R(0);
  if (d == 0) {
    acc += gterm<R, STEP>(xb[1], g, k, i, 2);
    acc += -gterm<R, STEP>(xb[2], g, k, i, 1);
  }
  else if (d == 1) {
    acc += -gterm<R, STEP>(xb[0], g, k, i, 2);
    acc += gterm<R, STEP>(xb[2], g, k, i, 0);
  }
  else {
    acc += gterm<R, STEP>(xb[0], g, k, i, 1);
    acc += -gterm<R, STEP>(xb[1], g, k, i, 0);
  }
  return acc;
}

// reverse of the D/E half-step at one point: E part (objective terms already
// in lambda_E, plus the gathered B-curl adjoints), then the D curl.  All
// loads of the three components first, then the arithmetic, then the stores.
template <typename R, bool FX, bool FY, bool FZ>
__device__ __forceinline__ void adj3_de_point(const Adj3Args<R> &a, const int k[3]) {
  const FusedArgs<R> &g = a.g;
  const int i = k[0] * g.s[0] + k[1] * g.s[1] + k[2];
  ShellFlags<R> F;
  band_flags<R, FX, FY, FZ>(g, k, F);
  const bool v[3] = {k[1] >= 1 && k[2] >= 1, k[0] >= 1 && k[2] >= 1, k[0] >= 1 && k[1] >= 1};
  R acc[3], lE[3], lD[3], ch[3], lfw[3], lfu[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const int ds = (d + 1) % 3, du = (d + 2) % 3;
    acc[d] = v[d] ? gather3<R, 1>(g, a.xbB, d, k, i) : R(0);
    lE[d] = v[d] ? a.lE[d][i] : R(0);
    lD[d] = v[d] ? a.lD[d][i] : R(0);
    ch[d] = v[d] ? a.chi[d][i] : R(0);
    lfw[d] = (v[d] && F.s1[d]) ? a.lfwE[d][i] : R(0);
    lfu[d] = (v[d] && F.s0[du]) ? a.lfuD[d][i] : R(0);
    (void)ds;
  }
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (!v[d]) continue;
    const R le = lE[d] + acc[d];
    R lam = lD[d];
    const int pw = 2 * k[d] + 1;
    R gsrc;
    if (F.s1[d]) {
      const R kk = g.kap[d][pw], ss = g.sig[d][pw];
      const R lfwn = lfw[d] + (kk + ss) * le;
      a.lfwE[d][i] = -(kk - ss) * le;
      a.lE[d][i] = le;
      lam += ch[d] * lfwn;
      gsrc = lfwn;
    }
    else {
      lam += ch[d] * le;
      a.lE[d][i] = R(0);
      gsrc = le;
    }
    if (a.rec[d]) {
      const int q0 = k[0] - a.dlo[0], q1 = k[1] - a.dlo[1], q2 = k[2] - a.dlo[2];
      if (q0 >= 0 && q0 < a.dn[0] && q1 >= 0 && q1 < a.dn[1] && q2 >= 0 && q2 < a.dn[2]) {
        const long long qi = ((long long)q0 * a.dn[1] + q1) * a.dn[2] + q2;
        a.grad[d][qi] += double(gsrc) * double(a.rec[d][qi]);
      }
    }
    // D_d at shift 1 along d, 0 elsewhere: dsig = d+1, dsigu = d+2 at 2k
    const int ds = (d + 1) % 3, du = (d + 2) % 3;
    const bool sg = F.s0[ds], su = F.s0[du];
    const AdjCurl3<R> o = adj3_curl<R>(g, a.c, sg, su, ds, 2 * k[ds], du, 2 * k[du], lfu[d], lam);
    a.lD[d][i] = o.lf;
    a.xbD[d][i] = o.xb;
    if (sg && su) a.lfuD[d][i] = o.lfu;
  }
}

// reverse of the B half-step at one point: H through f_w inside the slab
// along its own direction (gathered D-curl adjoints), then the B curl
template <typename R, bool FX, bool FY, bool FZ>
__device__ __forceinline__ void adj3_bh_point(const Adj3Args<R> &a, const int k[3]) {
  const FusedArgs<R> &g = a.g;
  const int i = k[0] * g.s[0] + k[1] * g.s[1] + k[2];
  ShellFlags<R> F;
  band_flags<R, FX, FY, FZ>(g, k, F);
  const bool v[3] = {k[0] >= 1, k[1] >= 1, k[2] >= 1};
  R gs[3], lB[3], lH[3], lfw[3], lfu[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const int du = (d + 2) % 3;
    gs[d] = v[d] ? gather3<R, -1>(g, a.xbD, d, k, i) : R(0);
    lB[d] = v[d] ? a.lB[d][i] : R(0);
    lH[d] = (v[d] && F.s0[d]) ? a.lH[d][i] : R(0);
    lfw[d] = (v[d] && F.s0[d]) ? a.lfwH[d][i] : R(0);
    lfu[d] = (v[d] && F.s1[du]) ? a.lfuB[d][i] : R(0);
  }
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (!v[d]) continue;
    R lam = lB[d];
    if (F.s0[d]) {
      const int pw = 2 * k[d];
      const R kk = g.kap[d][pw], ss = g.sig[d][pw];
      const R lh = lH[d] + gs[d];
      a.lH[d][i] = lh;
      lam += (kk + ss) * lh + lfw[d];
      a.lfwH[d][i] = -(kk - ss) * lh;
    }
    else
      lam += gs[d];
    // B_d at shift 0 along d, 1 elsewhere: dsig = d+1, dsigu = d+2 at 2k+1
    const int ds = (d + 1) % 3, du = (d + 2) % 3;
    const bool sg = F.s1[ds], su = F.s1[du];
    const AdjCurl3<R> o = adj3_curl<R>(g, a.c, sg, su, ds, 2 * k[ds] + 1, du, 2 * k[du] + 1, lfu[d], lam);
    a.lB[d][i] = o.lf;
    a.xbB[d][i] = o.xb;
    if (sg && su) a.lfuB[d][i] = o.lfu;
  }
}

template <typename R, bool FX, bool FY, bool FZ>
__global__ void __launch_bounds__(256, 8) adj3_de_band_kernel(const Adj3Args<R> a, const Band bd) {
  int k[3];
  if (band_coords(bd, k)) adj3_de_point<R, FX, FY, FZ>(a, k);
}

template <typename R, bool FX, bool FY, bool FZ>
__global__ void __launch_bounds__(256, 8) adj3_bh_band_kernel(const Adj3Args<R> a, const Band bd) {
  int k[3];
  if (band_coords(bd, k)) adj3_bh_point<R, FX, FY, FZ>(a, k);
}

} // namespace cuda_impl
} // namespace mfd
