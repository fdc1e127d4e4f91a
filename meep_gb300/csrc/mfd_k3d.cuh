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
