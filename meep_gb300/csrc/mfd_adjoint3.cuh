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

// adjoint of step_curl's branches for one component (adj_curl_core)
template <typename R>
__device__ __forceinline__ void adj3_curl(const FusedArgs<R> &g, R c, bool sg, bool su, int ds, int ps, int du,
                                          int pu, R *lf, R *lfu, R *xbar, int i, R lam) {
  R lfv, xb;
  if (!sg && !su) {
    lfv = lam;
    xb = -c * lam;
  }
  else if (!sg && su) {
    const R siu = g.siginv[du][pu], ku = g.kap[du][pu] - g.sig[du][pu];
    const R lt = lfu[i] + siu * lam;
    lfv = siu * ku * lam;
    xb = -c * lt;
  }
  else if (sg && !su) {
    const R si = g.siginv[ds][ps], ks = g.kap[ds][ps] - g.sig[ds][ps];
    lfv = ks * si * lam;
    xb = -c * si * lam;
  }
  else {
    const R si = g.siginv[ds][ps], ks = g.kap[ds][ps] - g.sig[ds][ps];
    const R siu = g.siginv[du][pu], ku = g.kap[du][pu] - g.sig[du][pu];
    const R lt = lfu[i] + siu * lam;
    lfv = siu * ku * lam;
    lfu[i] = ks * si * lt - siu * lam;
    xb = -c * si * lt;
  }
  lf[i] = lfv;
  xbar[i] = xb;
}

// reverse of the D/E half-step at one point: E part (objective terms already
// in lambda_E, plus the gathered B-curl adjoints), then the D curl
template <typename R, bool FX, bool FY, bool FZ>
__device__ __forceinline__ void adj3_de_point(const Adj3Args<R> &a, const int k[3]) {
  const FusedArgs<R> &g = a.g;
  const int i = k[0] * g.s[0] + k[1] * g.s[1] + k[2];
  ShellFlags<R> F;
  band_flags<R, FX, FY, FZ>(g, k, F);
  const bool v[3] = {k[1] >= 1 && k[2] >= 1, k[0] >= 1 && k[2] >= 1, k[0] >= 1 && k[1] >= 1};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (!v[d]) continue;
    R acc = R(0);
    if (d == 0) {
      acc += gterm<R, 1>(a.xbB[1], g, k, i, 2);
      acc += -gterm<R, 1>(a.xbB[2], g, k, i, 1);
    }
    else if (d == 1) {
      acc += -gterm<R, 1>(a.xbB[0], g, k, i, 2);
      acc += gterm<R, 1>(a.xbB[2], g, k, i, 0);
    }
    else {
      acc += gterm<R, 1>(a.xbB[0], g, k, i, 1);
      acc += -gterm<R, 1>(a.xbB[1], g, k, i, 0);
    }
    const R le = a.lE[d][i] + acc;
    R lam = a.lD[d][i];
    const int pw = 2 * k[d] + 1;
    R gsrc;
    if (F.s1[d]) {
      const R kk = g.kap[d][pw], ss = g.sig[d][pw];
      const R lfw = a.lfwE[d][i] + (kk + ss) * le;
      a.lfwE[d][i] = -(kk - ss) * le;
      a.lE[d][i] = le;
      lam += a.chi[d][i] * lfw;
      gsrc = lfw;
    }
    else {
      lam += a.chi[d][i] * le;
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
    adj3_curl<R>(g, a.c, F.s0[ds], F.s0[du], ds, 2 * k[ds], du, 2 * k[du], a.lD[d], a.lfuD[d], a.xbD[d], i, lam);
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
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (!v[d]) continue;
    R gsum = R(0);
    if (d == 0) {
      gsum += gterm<R, -1>(a.xbD[1], g, k, i, 2);
      gsum += -gterm<R, -1>(a.xbD[2], g, k, i, 1);
    }
    else if (d == 1) {
      gsum += -gterm<R, -1>(a.xbD[0], g, k, i, 2);
      gsum += gterm<R, -1>(a.xbD[2], g, k, i, 0);
    }
    else {
      gsum += gterm<R, -1>(a.xbD[0], g, k, i, 1);
      gsum += -gterm<R, -1>(a.xbD[1], g, k, i, 0);
    }
    R lam = a.lB[d][i];
    if (F.s0[d]) {
      const int pw = 2 * k[d];
      const R kk = g.kap[d][pw], ss = g.sig[d][pw];
      const R lh = a.lH[d][i] + gsum;
      a.lH[d][i] = lh;
      lam += (kk + ss) * lh + a.lfwH[d][i];
      a.lfwH[d][i] = -(kk - ss) * lh;
    }
    else
      lam += gsum;
    // B_d at shift 0 along d, 1 elsewhere: dsig = d+1, dsigu = d+2 at 2k+1
    const int ds = (d + 1) % 3, du = (d + 2) % 3;
    adj3_curl<R>(g, a.c, F.s1[ds], F.s1[du], ds, 2 * k[ds] + 1, du, 2 * k[du] + 1, a.lB[d], a.lfuB[d], a.xbB[d], i,
                 lam);
  }
}

template <typename R, bool FX, bool FY, bool FZ>
__global__ void __launch_bounds__(256) adj3_de_band_kernel(const Adj3Args<R> a, const Band bd) {
  int k[3];
  if (band_coords(bd, k)) adj3_de_point<R, FX, FY, FZ>(a, k);
}

template <typename R, bool FX, bool FY, bool FZ>
__global__ void __launch_bounds__(256) adj3_bh_band_kernel(const Adj3Args<R> a, const Band bd) {
  int k[3];
  if (band_coords(bd, k)) adj3_bh_point<R, FX, FY, FZ>(a, k);
}

} // namespace cuda_impl
} // namespace mfd
