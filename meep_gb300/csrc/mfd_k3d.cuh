// Hand-written 3-D interior kernels.  The interior box holds only points of
// the reference's interior chunk (no PML slab, no metal wall, H == B), so the
// updates are the plain branches of step_curl (src/step_generic.cpp:94-113)
// and step_update_EDHB (src/step_generic.cpp:769-777) plus the Lorentzian
// recurrence (src/susceptibility.cpp:249-255), with the operands spelled out:
//   B -= dtdx * curl E     (forward differences, strides +)
//   D -= dtdx * curl' H    (backward differences, strides negated)
//   E  = chi1inv * (D - sum P);  P, P_prev <- Lorentz/Drude update with W = E
// Grid: blockIdx.x,y tile z (32) and y (8), blockIdx.z is the x plane.
#pragma once

namespace mfd {
namespace cuda_impl {

struct IBox {
  int lo[3], n[3];
};

template <typename R, bool CND>
__global__ void __launch_bounds__(256) b3_interior_kernel(const FusedArgs<R> a, const IBox b) {
  const int k2 = b.lo[2] + blockIdx.x * 32 + threadIdx.x;
  const int k1 = b.lo[1] + blockIdx.y * 8 + threadIdx.y;
  const int k0 = b.lo[0] + blockIdx.z;
  if (k2 >= b.lo[2] + b.n[2] || k1 >= b.lo[1] + b.n[1]) return;
  const int sx = a.s[0], sy = a.s[1];
  const int i = k0 * sx + k1 * sy + k2;
  const R *__restrict__ Ex = a.e[0];
  const R *__restrict__ Ey = a.e[1];
  const R *__restrict__ Ez = a.e[2];
  const R ex = Ex[i], exy = Ex[i + sy], exz = Ex[i + 1];
  const R ey = Ey[i], eyx = Ey[i + sx], eyz = Ey[i + 1];
  const R ez = Ez[i], ezx = Ez[i + sx], ezy = Ez[i + sy];
  const R bx = a.b[0][i], by = a.b[1][i], bz = a.b[2][i];
  const R Xx = (ezy - ez) + ey - eyz;
  const R Xy = (exz - ex) + ez - ezx;
  const R Xz = (eyx - ey) + ex - exy;
  const R dtdx = a.dtdx;
  R nbx, nby, nbz;
  if (CND) {
    const R one = R(1);
    nbx = a.cnd[3][0] ? ((one - a.dt2 * a.cnd[3][0][i]) * bx - dtdx * Xx) * a.cndinv[3][0][i] : bx - dtdx * Xx;
    nby = a.cnd[3][1] ? ((one - a.dt2 * a.cnd[3][1][i]) * by - dtdx * Xy) * a.cndinv[3][1][i] : by - dtdx * Xy;
    nbz = a.cnd[3][2] ? ((one - a.dt2 * a.cnd[3][2][i]) * bz - dtdx * Xz) * a.cndinv[3][2][i] : bz - dtdx * Xz;
  }
  else {
    nbx = bx - dtdx * Xx;
    nby = by - dtdx * Xy;
    nbz = bz - dtdx * Xz;
  }
  a.b[0][i] = nbx;
  a.b[1][i] = nby;
  a.b[2][i] = nbz;
}

template <typename R>
__device__ __forceinline__ R e_from_d(const FusedArgs<R> &a, int dc, int i, R dn, int npoles) {
  R gs = dn;
  for (int q = 0; q < npoles; q++)
    if (a.P[q][dc]) gs -= a.P[q][dc][i];
  const R e = gs * a.chi[dc][i];
  for (int q = 0; q < npoles; q++)
    if (a.P[q][dc]) {
      const R pcur = a.P[q][dc][i];
      a.P[q][dc][i] = a.pg1inv[q] * (pcur * (R(2) - a.pw0d[q]) - a.pg1[q] * a.PP[q][dc][i] +
                                     a.pw0[q] * (a.ps[q][dc][i] * e));
      a.PP[q][dc][i] = pcur;
    }
  return e;
}

template <typename R, bool CND, bool POLES>
__global__ void __launch_bounds__(256) de3_interior_kernel(const FusedArgs<R> a, const IBox b) {
  const int k2 = b.lo[2] + blockIdx.x * 32 + threadIdx.x;
  const int k1 = b.lo[1] + blockIdx.y * 8 + threadIdx.y;
  const int k0 = b.lo[0] + blockIdx.z;
  if (k2 >= b.lo[2] + b.n[2] || k1 >= b.lo[1] + b.n[1]) return;
  const int sx = a.s[0], sy = a.s[1];
  const int i = k0 * sx + k1 * sy + k2;
  const R *__restrict__ Hx = a.b[0]; // H == B in the interior chunk
  const R *__restrict__ Hy = a.b[1];
  const R *__restrict__ Hz = a.b[2];
  const R hx = Hx[i], hxy = Hx[i - sy], hxz = Hx[i - 1];
  const R hy = Hy[i], hyx = Hy[i - sx], hyz = Hy[i - 1];
  const R hz = Hz[i], hzx = Hz[i - sx], hzy = Hz[i - sy];
  const R dx = a.d[0][i], dy = a.d[1][i], dz = a.d[2][i];
  const R cx = a.chi[0][i], cy = a.chi[1][i], cz = a.chi[2][i];
  const R Xx = (hzy - hz) + hy - hyz;
  const R Xy = (hxz - hx) + hz - hzx;
  const R Xz = (hyx - hy) + hx - hxy;
  const R dtdx = a.dtdx;
  R ndx, ndy, ndz;
  if (CND) {
    const R one = R(1);
    ndx = a.cnd[2][0] ? ((one - a.dt2 * a.cnd[2][0][i]) * dx - dtdx * Xx) * a.cndinv[2][0][i] : dx - dtdx * Xx;
    ndy = a.cnd[2][1] ? ((one - a.dt2 * a.cnd[2][1][i]) * dy - dtdx * Xy) * a.cndinv[2][1][i] : dy - dtdx * Xy;
    ndz = a.cnd[2][2] ? ((one - a.dt2 * a.cnd[2][2][i]) * dz - dtdx * Xz) * a.cndinv[2][2][i] : dz - dtdx * Xz;
  }
  else {
    ndx = dx - dtdx * Xx;
    ndy = dy - dtdx * Xy;
    ndz = dz - dtdx * Xz;
  }
  a.d[0][i] = ndx;
  a.d[1][i] = ndy;
  a.d[2][i] = ndz;
  if (POLES) {
    a.e[0][i] = e_from_d(a, 0, i, ndx, a.npoles);
    a.e[1][i] = e_from_d(a, 1, i, ndy, a.npoles);
    a.e[2][i] = e_from_d(a, 2, i, ndz, a.npoles);
  }
  else {
    a.e[0][i] = ndx * cx;
    a.e[1][i] = ndy * cy;
    a.e[2][i] = ndz * cz;
  }
}

} // namespace cuda_impl
} // namespace mfd

namespace mfd {
namespace cuda_impl {

// ------------------------------------------------------------ PML shell
// Points of the shell (PML slabs, metal walls, chunk boundaries) take the
// general branches of step_curl / step_update_EDHB.  Each component's branch
// is chosen from the chunk region of its own Yee position, exactly as the
// reference picks dsig / dsigu / dsigw per chunk (src/step_db.cpp:54-60,
// src/update_eh.cpp:159-160).  Loads of every component are issued before any
// store.

template <typename R> struct CurlRes {
  R f, fu, fc;
  bool wfu, wfc;
};

// step_curl branches for one point (src/step_generic.cpp:94-248)
template <typename R>
__device__ __forceinline__ CurlRes<R> curl_general(R fold, R X, R dtdx, R dt2, bool sg, bool su, bool hc,
                                                   const R *sig_s, const R *kap_s, const R *si_s, int ps,
                                                   const R *sig_u, const R *kap_u, const R *si_u, int pu,
                                                   const R *fu, const R *fcnd, const R *cnd,
                                                   const R *cndinv, int i) {
  CurlRes<R> o;
  o.wfu = o.wfc = false;
  o.fu = o.fc = R(0);
  const R one = R(1);
  if (!sg) {
    if (!su) {
      o.f = hc ? ((one - dt2 * cnd[i]) * fold - dtdx * X) * cndinv[i] : fold - dtdx * X;
      return o;
    }
    const R fprev = fu[i];
    const R fun = hc ? ((one - dt2 * cnd[i]) * fprev - dtdx * X) * cndinv[i] : fprev - dtdx * X;
    o.fu = fun;
    o.wfu = true;
    o.f = si_u[pu] * ((kap_u[pu] - sig_u[pu]) * fold + fun - fprev);
    return o;
  }
  const R ks = kap_s[ps] - sig_s[ps], si = si_s[ps];
  if (!su) {
    if (hc) {
      const R fcp = fcnd[i];
      const R fcn = ((one - dt2 * cnd[i]) * fcp - dtdx * X) * cndinv[i];
      o.fc = fcn;
      o.wfc = true;
      o.f = (ks * fold + (fcn - fcp)) * si;
    }
    else
      o.f = (ks * fold - dtdx * X) * si;
    return o;
  }
  const R fprev = fu[i];
  R fun;
  if (hc) {
    const R fcp = fcnd[i];
    const R fcn = ((one - dt2 * cnd[i]) * fcp - dtdx * X) * cndinv[i];
    o.fc = fcn;
    o.wfc = true;
    fun = (ks * fprev + (fcn - fcp)) * si;
  }
  else
    fun = (ks * fprev - dtdx * X) * si;
  o.fu = fun;
  o.wfu = true;
  o.f = si_u[pu] * ((kap_u[pu] - sig_u[pu]) * fold + fun - fprev);
  return o;
}

template <typename R> struct ShellFlags {
  int r0[3], r1[3]; // chunk region of positions 2k and 2k+1 along X, Y, Z
  bool s0[3], s1[3];
};

template <typename R> __device__ __forceinline__ void shell_flags(const FusedArgs<R> &a, const int k[3], ShellFlags<R> &f) {
#pragma unroll
  for (int d = 0; d < 3; d++) {
    f.r0[d] = fregion(a, d, 2 * k[d]);
    f.r1[d] = fregion(a, d, 2 * k[d] + 1);
    f.s0[d] = a.pml[d] && f.r0[d] != 1;
    f.s1[d] = a.pml[d] && f.r1[d] != 1;
  }
}

// does the chunk holding this component position carry a conductivity array
__device__ __forceinline__ bool chunk_has(unsigned mask, int rx, int ry, int rz) {
  return (mask >> (rx * 9 + ry * 3 + rz)) & 1u;
}

template <typename R>
__global__ void __launch_bounds__(256) b3_shell_kernel(const FusedArgs<R> a, const BoxList L) {
  int k[3];
  if (!box_coords<3>(L, k)) return;
  const int sx = a.s[0], sy = a.s[1];
  const int i = k[0] * sx + k[1] * sy + k[2];
  ShellFlags<R> F;
  shell_flags(a, k, F);
  // the low wall point (k = 0) of a component with shift 0 is not advanced
  const bool vx = k[0] >= 1, vy = k[1] >= 1, vz = k[2] >= 1;
  const R *Ex = a.e[0], *Ey = a.e[1], *Ez = a.e[2];
  const R ex = Ex[i], exy = Ex[i + sy], exz = Ex[i + 1];
  const R ey = Ey[i], eyx = Ey[i + sx], eyz = Ey[i + 1];
  const R ez = Ez[i], ezx = Ez[i + sx], ezy = Ez[i + sy];
  const R bx = a.b[0][i], by = a.b[1][i], bz = a.b[2][i];
  const R Xx = (ezy - ez) + ey - eyz;
  const R Xy = (exz - ex) + ez - ezx;
  const R Xz = (eyx - ey) + ex - exy;
  const R dtdx = a.dtdx, dt2 = a.dt2;
  const int p0x = 2 * k[0], p1x = p0x + 1, p0y = 2 * k[1], p1y = p0y + 1, p0z = 2 * k[2], p1z = p0z + 1;
  // Bx at (0,1,1): dsig = Y, dsigu = Z
  bool hcx = a.cnd[3][0] != nullptr, hcy = a.cnd[3][1] != nullptr, hcz = a.cnd[3][2] != nullptr;
  if (hcx && F.s1[1]) hcx = chunk_has(a.cond_chunks[3][0], F.r0[0], F.r1[1], F.r1[2]);
  if (hcy && F.s1[2]) hcy = chunk_has(a.cond_chunks[3][1], F.r1[0], F.r0[1], F.r1[2]);
  if (hcz && F.s1[0]) hcz = chunk_has(a.cond_chunks[3][2], F.r1[0], F.r1[1], F.r0[2]);
  const CurlRes<R> cx = curl_general(bx, Xx, dtdx, dt2, F.s1[1], F.s1[2], hcx, a.sig[1], a.kap[1], a.siginv[1], p1y,
                                     a.sig[2], a.kap[2], a.siginv[2], p1z, a.fu[3][0], a.fcnd[3][0], a.cnd[3][0],
                                     a.cndinv[3][0], i);
  // By at (1,0,1): dsig = Z, dsigu = X
  const CurlRes<R> cy = curl_general(by, Xy, dtdx, dt2, F.s1[2], F.s1[0], hcy, a.sig[2], a.kap[2], a.siginv[2], p1z,
                                     a.sig[0], a.kap[0], a.siginv[0], p1x, a.fu[3][1], a.fcnd[3][1], a.cnd[3][1],
                                     a.cndinv[3][1], i);
  // Bz at (1,1,0): dsig = X, dsigu = Y
  const CurlRes<R> cz = curl_general(bz, Xz, dtdx, dt2, F.s1[0], F.s1[1], hcz, a.sig[0], a.kap[0], a.siginv[0], p1x,
                                     a.sig[1], a.kap[1], a.siginv[1], p1y, a.fu[3][2], a.fcnd[3][2], a.cnd[3][2],
                                     a.cndinv[3][2], i);
  // H through f_w inside the slab along its own direction (shift 0 there)
  const bool hx = a.fuse_h && F.s0[0] && vx, hy = a.fuse_h && F.s0[1] && vy, hz = a.fuse_h && F.s0[2] && vz;
  R nhx = R(0), nhy = R(0), nhz = R(0), fwx = R(0), fwy = R(0), fwz = R(0);
  if (hx) {
    const R fwprev = a.fw[1][0][i], kk = a.kap[0][p0x], ss = a.sig[0][p0x];
    nhx = a.h[0][i] + ((kk + ss) * cx.f - (kk - ss) * fwprev);
  }
  if (hy) {
    const R fwprev = a.fw[1][1][i], kk = a.kap[1][p0y], ss = a.sig[1][p0y];
    nhy = a.h[1][i] + ((kk + ss) * cy.f - (kk - ss) * fwprev);
  }
  if (hz) {
    const R fwprev = a.fw[1][2][i], kk = a.kap[2][p0z], ss = a.sig[2][p0z];
    nhz = a.h[2][i] + ((kk + ss) * cz.f - (kk - ss) * fwprev);
  }
  fwx = cx.f;
  fwy = cy.f;
  fwz = cz.f;
  if (vx) {
    a.b[0][i] = cx.f;
    if (cx.wfu) a.fu[3][0][i] = cx.fu;
    if (cx.wfc) a.fcnd[3][0][i] = cx.fc;
    if (hx) {
      a.fw[1][0][i] = fwx;
      a.h[0][i] = nhx;
    }
  }
  if (vy) {
    a.b[1][i] = cy.f;
    if (cy.wfu) a.fu[3][1][i] = cy.fu;
    if (cy.wfc) a.fcnd[3][1][i] = cy.fc;
    if (hy) {
      a.fw[1][1][i] = fwy;
      a.h[1][i] = nhy;
    }
  }
  if (vz) {
    a.b[2][i] = cz.f;
    if (cz.wfu) a.fu[3][2][i] = cz.fu;
    if (cz.wfc) a.fcnd[3][2][i] = cz.fc;
    if (hz) {
      a.fw[1][2][i] = fwz;
      a.h[2][i] = nhz;
    }
  }
}

// E from the new D (f_minus_p = D - P), f_w inside the slab along its own
// direction, then the poles with W = f_w or E (update_eh + update_pols).
template <typename R> struct EShell {
  R e, fw;
  bool wfw;
};

template <typename R>
__device__ __forceinline__ EShell<R> e_general(const FusedArgs<R> &a, int dc, int i, R dn, bool slabw, int pw) {
  R gs = dn;
  for (int q = 0; q < a.npoles; q++)
    if (a.P[q][dc]) gs -= a.P[q][dc][i];
  const R us = a.chi[dc][i];
  EShell<R> o;
  R W;
  if (slabw) {
    const R fwprev = a.fw[0][dc][i], kk = a.kap[dc][pw], ss = a.sig[dc][pw];
    const R fwn = (gs * us);
    o.fw = fwn;
    o.wfw = true;
    o.e = a.e[dc][i] + ((kk + ss) * fwn - (kk - ss) * fwprev);
    W = fwn;
  }
  else {
    o.e = (gs * us);
    o.fw = R(0);
    o.wfw = false;
    W = o.e;
  }
  for (int q = 0; q < a.npoles; q++)
    if (a.P[q][dc]) {
      const R pcur = a.P[q][dc][i];
      a.P[q][dc][i] = a.pg1inv[q] * (pcur * (R(2) - a.pw0d[q]) - a.pg1[q] * a.PP[q][dc][i] +
                                     a.pw0[q] * (a.ps[q][dc][i] * W));
      a.PP[q][dc][i] = pcur;
    }
  return o;
}

template <typename R>
__global__ void __launch_bounds__(256) de3_shell_kernel(const FusedArgs<R> a, const BoxList L) {
  int k[3];
  if (!box_coords<3>(L, k)) return;
  const int sx = a.s[0], sy = a.s[1];
  const int i = k[0] * sx + k[1] * sy + k[2];
  ShellFlags<R> F;
  shell_flags(a, k, F);
  // D components sit at shift 1 along their own direction, 0 elsewhere:
  // Dx (1,0,0) needs k_y, k_z >= 1; Dy needs k_x, k_z >= 1; Dz needs k_x, k_y >= 1
  const bool vx = k[1] >= 1 && k[2] >= 1, vy = k[0] >= 1 && k[2] >= 1, vz = k[0] >= 1 && k[1] >= 1;
  // H read where the owning chunk keeps a separate H (slab along its own
  // direction, shift 0 there), B elsewhere
  const R *Hx = F.s0[0] ? a.h[0] : a.b[0];
  const R *Hy = F.s0[1] ? a.h[1] : a.b[1];
  const R *Hz = F.s0[2] ? a.h[2] : a.b[2];
  // backward neighbours at k = 0 belong only to components that are not
  // advanced there (low metal wall); clamp them onto the point itself so no
  // load leaves the array
  const int mx = k[0] >= 1 ? sx : 0, my = k[1] >= 1 ? sy : 0, mz = k[2] >= 1 ? 1 : 0;
  const R hx = Hx[i], hxy = Hx[i - my], hxz = Hx[i - mz];
  const R hy = Hy[i], hyx = Hy[i - mx], hyz = Hy[i - mz];
  const R hz = Hz[i], hzx = Hz[i - mx], hzy = Hz[i - my];
  const R dx = a.d[0][i], dy = a.d[1][i], dz = a.d[2][i];
  const R Xx = (hzy - hz) + hy - hyz;
  const R Xy = (hxz - hx) + hz - hzx;
  const R Xz = (hyx - hy) + hx - hxy;
  const R dtdx = a.dtdx, dt2 = a.dt2;
  const int p0x = 2 * k[0], p1x = p0x + 1, p0y = 2 * k[1], p1y = p0y + 1, p0z = 2 * k[2], p1z = p0z + 1;
  bool hcx = a.cnd[2][0] != nullptr, hcy = a.cnd[2][1] != nullptr, hcz = a.cnd[2][2] != nullptr;
  // Dx (1,0,0): dsig = Y (shift 0), dsigu = Z (shift 0)
  if (hcx && F.s0[1]) hcx = chunk_has(a.cond_chunks[2][0], F.r1[0], F.r0[1], F.r0[2]);
  // Dy (0,1,0): dsig = Z, dsigu = X
  if (hcy && F.s0[2]) hcy = chunk_has(a.cond_chunks[2][1], F.r0[0], F.r1[1], F.r0[2]);
  // Dz (0,0,1): dsig = X, dsigu = Y
  if (hcz && F.s0[0]) hcz = chunk_has(a.cond_chunks[2][2], F.r0[0], F.r0[1], F.r1[2]);
  const CurlRes<R> cx = curl_general(dx, Xx, dtdx, dt2, F.s0[1], F.s0[2], hcx, a.sig[1], a.kap[1], a.siginv[1], p0y,
                                     a.sig[2], a.kap[2], a.siginv[2], p0z, a.fu[2][0], a.fcnd[2][0], a.cnd[2][0],
                                     a.cndinv[2][0], i);
  const CurlRes<R> cy = curl_general(dy, Xy, dtdx, dt2, F.s0[2], F.s0[0], hcy, a.sig[2], a.kap[2], a.siginv[2], p0z,
                                     a.sig[0], a.kap[0], a.siginv[0], p0x, a.fu[2][1], a.fcnd[2][1], a.cnd[2][1],
                                     a.cndinv[2][1], i);
  const CurlRes<R> cz = curl_general(dz, Xz, dtdx, dt2, F.s0[0], F.s0[1], hcz, a.sig[0], a.kap[0], a.siginv[0], p0x,
                                     a.sig[1], a.kap[1], a.siginv[1], p0y, a.fu[2][2], a.fcnd[2][2], a.cnd[2][2],
                                     a.cndinv[2][2], i);
  // E components share the D positions: f_w slab along their own direction at shift 1
  if (vx) {
    const EShell<R> ox = e_general(a, 0, i, cx.f, F.s1[0], p1x);
    a.d[0][i] = cx.f;
    if (cx.wfu) a.fu[2][0][i] = cx.fu;
    if (cx.wfc) a.fcnd[2][0][i] = cx.fc;
    a.e[0][i] = ox.e;
    if (ox.wfw) a.fw[0][0][i] = ox.fw;
  }
  if (vy) {
    const EShell<R> oy = e_general(a, 1, i, cy.f, F.s1[1], p1y);
    a.d[1][i] = cy.f;
    if (cy.wfu) a.fu[2][1][i] = cy.fu;
    if (cy.wfc) a.fcnd[2][1][i] = cy.fc;
    a.e[1][i] = oy.e;
    if (oy.wfw) a.fw[0][1][i] = oy.fw;
  }
  if (vz) {
    const EShell<R> oz = e_general(a, 2, i, cz.f, F.s1[2], p1z);
    a.d[2][i] = cz.f;
    if (cz.wfu) a.fu[2][2][i] = cz.fu;
    if (cz.wfc) a.fcnd[2][2][i] = cz.fc;
    a.e[2][i] = oz.e;
    if (oz.wfw) a.fw[0][2][i] = oz.fw;
  }
}

} // namespace cuda_impl
} // namespace mfd
