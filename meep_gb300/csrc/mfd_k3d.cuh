// Hand-written 3-D one-point kernels over bands of the grid.  A band is a
// box whose x, y and z ranges are either a contiguous run or the two slabs
// outside an interior run; the launch maps blockIdx.z to x, blockIdx.y and
// threadIdx.y to y, blockIdx.x and threadIdx.x to z (unit stride), so every
// warp is a run of consecutive z points of one row.
//
// The per-point code takes the general branches of step_curl /
// step_update_EDHB; each component's branch is chosen from the chunk region
// of its own Yee position, exactly as the reference picks dsig / dsigu /
// dsigw per chunk (src/step_db.cpp:54-60, src/update_eh.cpp:159-160).  The
// band kernels are templated on which directions can hold PML slab points:
// for the others the flags are compile-time "interior" and their branches
// vanish.
#pragma once

namespace mfd {
namespace cuda_impl {

// k = t + (t < split ? a0 : a1) for t < n: a contiguous run (split = n) or
// the two slabs around an interior run
struct Span {
  int n, split, a0, a1;
};
struct Band {
  Span s[3];
};

template <typename R> struct CurlRes {
  R f, fu, fc;
  bool wfu, wfc;
};

// the field-sized operands of one component's step_curl branch, loaded up
// front with predicated loads: no branch separates the loads of the three
// components of a point, so they are all in flight together (loads inside
// the branches would wait for each other, one memory round trip per branch)
template <typename R> struct CurlIn {
  R fu, fc, cnd, cndinv;
};
template <typename R>
__device__ __forceinline__ CurlIn<R> curl_in(bool sg, bool su, bool hc, const R *fu, const R *fcnd, const R *cnd,
                                             const R *cndinv, int i) {
  CurlIn<R> v;
  v.fu = su ? fu[i] : R(0);
  v.fc = (sg && hc) ? fcnd[i] : R(0);
  v.cnd = hc ? cnd[i] : R(0);
  v.cndinv = hc ? cndinv[i] : R(0);
  return v;
}

// step_curl branches for one point (src/step_generic.cpp:94-248)
template <typename R>
__device__ __forceinline__ CurlRes<R> curl_general(R fold, R X, R dtdx, R dt2, bool sg, bool su, bool hc,
                                                   const R *sig_s, const R *kap_s, const R *si_s, int ps,
                                                   const R *sig_u, const R *kap_u, const R *si_u, int pu,
                                                   const CurlIn<R> &v) {
  CurlRes<R> o;
  o.wfu = o.wfc = false;
  o.fu = o.fc = R(0);
  const R one = R(1);
  if (!sg) {
    if (!su) {
      o.f = hc ? ((one - dt2 * v.cnd) * fold - dtdx * X) * v.cndinv : fold - dtdx * X;
      return o;
    }
    const R fprev = v.fu;
    const R fun = hc ? ((one - dt2 * v.cnd) * fprev - dtdx * X) * v.cndinv : fprev - dtdx * X;
    o.fu = fun;
    o.wfu = true;
    o.f = si_u[pu] * ((kap_u[pu] - sig_u[pu]) * fold + fun - fprev);
    return o;
  }
  const R ks = kap_s[ps] - sig_s[ps], si = si_s[ps];
  if (!su) {
    if (hc) {
      const R fcp = v.fc;
      const R fcn = ((one - dt2 * v.cnd) * fcp - dtdx * X) * v.cndinv;
      o.fc = fcn;
      o.wfc = true;
      o.f = (ks * fold + (fcn - fcp)) * si;
    }
    else
      o.f = (ks * fold - dtdx * X) * si;
    return o;
  }
  const R fprev = v.fu;
  R fun;
  if (hc) {
    const R fcp = v.fc;
    const R fcn = ((one - dt2 * v.cnd) * fcp - dtdx * X) * v.cndinv;
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

// flags of the directions that can hold slab points (FX, FY, FZ); the others
// are interior: middle chunk region, no slab
template <typename R, bool FX, bool FY, bool FZ>
__device__ __forceinline__ void band_flags(const FusedArgs<R> &a, const int k[3], ShellFlags<R> &f) {
  constexpr bool fl[3] = {FX, FY, FZ};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (fl[d]) {
      f.r0[d] = fregion(a, d, 2 * k[d]);
      f.r1[d] = fregion(a, d, 2 * k[d] + 1);
      f.s0[d] = a.pml[d] && f.r0[d] != 1;
      f.s1[d] = a.pml[d] && f.r1[d] != 1;
    }
    else {
      f.r0[d] = f.r1[d] = 1;
      f.s0[d] = f.s1[d] = false;
    }
  }
}

// point of this thread; false past the end of the band
__device__ __forceinline__ bool band_coords(const Band &bd, int k[3]) {
  const int t[3] = {(int)blockIdx.z, (int)(blockIdx.y * blockDim.y + threadIdx.y),
                    (int)(blockIdx.x * blockDim.x + threadIdx.x)};
  if (t[1] >= bd.s[1].n || t[2] >= bd.s[2].n) return false;
#pragma unroll
  for (int d = 0; d < 3; d++)
    k[d] = t[d] + (t[d] < bd.s[d].split ? bd.s[d].a0 : bd.s[d].a1);
  return true;
}

// does the chunk holding this component position carry a conductivity array
__device__ __forceinline__ bool chunk_has(unsigned mask, int rx, int ry, int rz) {
  return (mask >> (rx * 9 + ry * 3 + rz)) & 1u;
}

// activity bits of the row segment holding point k (FusedArgs::amask)
constexpr int AM_DCOND = 12, AM_BCOND = 15;
template <typename R> __device__ __forceinline__ unsigned seg_active(const FusedArgs<R> &a, const int k[3]) {
  if (a.am_all) return a.am_all;
  return a.amask ? __ldg(a.amask + ((size_t)k[0] * a.mext1 + k[1]) * a.mnseg + (k[2] >> 5)) : ~0u;
}
template <typename R>
__device__ __forceinline__ bool pole_on(const FusedArgs<R> &a, unsigned am, int q, int dc) {
  return q < a.npoles && a.P[q][dc] && ((am >> (3 * q + dc)) & 1u);
}

// B -= dtdx * curl E with PML / conductivity branches, then H inside the
// slab along its own direction (update_eh through f_w)
template <typename R, bool CND, bool FX, bool FY, bool FZ>
__device__ __forceinline__ void b3_point(const FusedArgs<R> &a, const int k[3]) {
  const int sx = a.s[0], sy = a.s[1];
  const int i = k[0] * sx + k[1] * sy + k[2];
  ShellFlags<R> F;
  band_flags<R, FX, FY, FZ>(a, k, F);
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
  bool hcx = CND && a.cnd[3][0] != nullptr, hcy = CND && a.cnd[3][1] != nullptr, hcz = CND && a.cnd[3][2] != nullptr;
  const unsigned am = CND ? seg_active(a, k) : 0u;
  if (hcx) hcx = F.s1[1] ? chunk_has(a.cond_chunks[3][0], F.r0[0], F.r1[1], F.r1[2]) : ((am >> (AM_BCOND + 0)) & 1u);
  if (hcy) hcy = F.s1[2] ? chunk_has(a.cond_chunks[3][1], F.r1[0], F.r0[1], F.r1[2]) : ((am >> (AM_BCOND + 1)) & 1u);
  if (hcz) hcz = F.s1[0] ? chunk_has(a.cond_chunks[3][2], F.r1[0], F.r1[1], F.r0[2]) : ((am >> (AM_BCOND + 2)) & 1u);
  // every field-sized operand of the point before any branch
  const CurlIn<R> inx = curl_in(F.s1[1], F.s1[2], hcx, a.fu[3][0], a.fcnd[3][0], a.cnd[3][0], a.cndinv[3][0], i);
  const CurlIn<R> iny = curl_in(F.s1[2], F.s1[0], hcy, a.fu[3][1], a.fcnd[3][1], a.cnd[3][1], a.cndinv[3][1], i);
  const CurlIn<R> inz = curl_in(F.s1[0], F.s1[1], hcz, a.fu[3][2], a.fcnd[3][2], a.cnd[3][2], a.cndinv[3][2], i);
  // H through f_w inside the slab along its own direction (shift 0 there)
  const bool hx = a.fuse_h && F.s0[0] && vx, hy = a.fuse_h && F.s0[1] && vy, hz = a.fuse_h && F.s0[2] && vz;
  const R fwx0 = hx ? a.fw[1][0][i] : R(0), hx0 = hx ? a.h[0][i] : R(0);
  const R fwy0 = hy ? a.fw[1][1][i] : R(0), hy0 = hy ? a.h[1][i] : R(0);
  const R fwz0 = hz ? a.fw[1][2][i] : R(0), hz0 = hz ? a.h[2][i] : R(0);
  const CurlRes<R> cx = curl_general(bx, Xx, dtdx, dt2, F.s1[1], F.s1[2], hcx, a.sig[1], a.kap[1], a.siginv[1], p1y,
                                     a.sig[2], a.kap[2], a.siginv[2], p1z, inx);
  // By at (1,0,1): dsig = Z, dsigu = X
  const CurlRes<R> cy = curl_general(by, Xy, dtdx, dt2, F.s1[2], F.s1[0], hcy, a.sig[2], a.kap[2], a.siginv[2], p1z,
                                     a.sig[0], a.kap[0], a.siginv[0], p1x, iny);
  // Bz at (1,1,0): dsig = X, dsigu = Y
  const CurlRes<R> cz = curl_general(bz, Xz, dtdx, dt2, F.s1[0], F.s1[1], hcz, a.sig[0], a.kap[0], a.siginv[0], p1x,
                                     a.sig[1], a.kap[1], a.siginv[1], p1y, inz);
  R nhx = R(0), nhy = R(0), nhz = R(0), fwx = R(0), fwy = R(0), fwz = R(0);
  if (hx) {
    const R kk = a.kap[0][p0x], ss = a.sig[0][p0x];
    nhx = hx0 + ((kk + ss) * cx.f - (kk - ss) * fwx0);
  }
  if (hy) {
    const R kk = a.kap[1][p0y], ss = a.sig[1][p0y];
    nhy = hy0 + ((kk + ss) * cy.f - (kk - ss) * fwy0);
  }
  if (hz) {
    const R kk = a.kap[2][p0z], ss = a.sig[2][p0z];
    nhz = hz0 + ((kk + ss) * cz.f - (kk - ss) * fwz0);
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
  R pn[MAX_POLES], pc[MAX_POLES]; // new and current P of each pole
};

// everything loaded and computed, nothing stored (so the loads of all three
// components are in flight together)
template <typename R, bool POLES>
__device__ __forceinline__ EShell<R> e_general(const FusedArgs<R> &a, int dc, int i, R dn, bool slabw, int pw,
                                               unsigned am) {
  EShell<R> o;
  R gs = dn;
  if (POLES) {
#pragma unroll
    for (int q = 0; q < MAX_POLES; q++)
      if (pole_on(a, am, q, dc)) {
        o.pc[q] = a.P[q][dc][i];
        gs -= o.pc[q];
      }
  }
  const R us = a.chi[dc][i];
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
  if (POLES) {
#pragma unroll
    for (int q = 0; q < MAX_POLES; q++)
      if (pole_on(a, am, q, dc))
        o.pn[q] = a.pg1inv[q] * (o.pc[q] * (R(2) - a.pw0d[q]) - a.pg1[q] * a.PP[q][dc][i] +
                                 a.pw0[q] * (a.ps[q][dc][i] * W));
  }
  return o;
}

template <typename R, bool POLES>
__device__ __forceinline__ void e_store(const FusedArgs<R> &a, int dc, int i, const EShell<R> &o, unsigned am) {
  a.e[dc][i] = o.e;
  if (o.wfw) a.fw[0][dc][i] = o.fw;
  if (POLES) {
#pragma unroll
    for (int q = 0; q < MAX_POLES; q++)
      if (pole_on(a, am, q, dc)) {
        a.P[q][dc][i] = o.pn[q];
        a.PP[q][dc][i] = o.pc[q];
      }
  }
}

// the E operands of one component without poles, loaded up front
template <typename R> struct EIn {
  R us, fw, e;
};
template <typename R>
__device__ __forceinline__ EIn<R> e_in(const FusedArgs<R> &a, int dc, int i, bool v, bool slabw) {
  EIn<R> o;
  o.us = v ? a.chi[dc][i] : R(0);
  o.fw = (v && slabw) ? a.fw[0][dc][i] : R(0);
  o.e = (v && slabw) ? a.e[dc][i] : R(0);
  return o;
}
// e_general without poles, from preloaded operands (same arithmetic)
template <typename R>
__device__ __forceinline__ EShell<R> e_from(const FusedArgs<R> &a, int dc, R dn, bool slabw, int pw, const EIn<R> &in) {
  EShell<R> o;
  if (slabw) {
    const R kk = a.kap[dc][pw], ss = a.sig[dc][pw];
    const R fwn = (dn * in.us);
    o.fw = fwn;
    o.wfw = true;
    o.e = in.e + ((kk + ss) * fwn - (kk - ss) * in.fw);
  }
  else {
    o.e = (dn * in.us);
    o.fw = R(0);
    o.wfw = false;
  }
  return o;
}

// The E operands of one component with NP poles held in registers (NP = 1
// or 2), loaded with the curl operands before any store so that every load
// of the point is in flight at once: chi, E and f_w in the component's own
// slab, and for each pole active in the row segment P, P_prev and sigma.
template <typename R, int NP> struct EPoleIn {
  R us, fw, e;
  R p[NP], pp[NP], s[NP];
  bool on[NP];
};
template <typename R, int NP>
__device__ __forceinline__ EPoleIn<R, NP> epole_in(const FusedArgs<R> &a, int dc, int i, bool v, bool slabw,
                                                   unsigned am) {
  EPoleIn<R, NP> o;
  o.us = v ? a.chi[dc][i] : R(0);
  o.fw = (v && slabw) ? a.fw[0][dc][i] : R(0);
  o.e = (v && slabw) ? a.e[dc][i] : R(0);
#pragma unroll
  for (int q = 0; q < NP; q++) {
    o.on[q] = v && pole_on(a, am, q, dc);
    o.p[q] = o.on[q] ? a.P[q][dc][i] : R(0);
    o.pp[q] = o.on[q] ? a.PP[q][dc][i] : R(0);
    o.s[q] = o.on[q] ? a.ps[q][dc][i] : R(0);
  }
  return o;
}
// E = chi (D - sum P) (through f_w in the slab), then the new P of each pole
// with W = f_w or E: the arithmetic of e_general in the same order
template <typename R, int NP> struct EPoleOut {
  R e, fw;
  bool wfw;
  R pn[NP];
};
template <typename R, int NP>
__device__ __forceinline__ EPoleOut<R, NP> epole_from(const FusedArgs<R> &a, int dc, R dn, bool slabw, int pw,
                                                      const EPoleIn<R, NP> &in) {
  EPoleOut<R, NP> o;
  R gs = dn;
#pragma unroll
  for (int q = 0; q < NP; q++)
    if (in.on[q]) gs -= in.p[q];
  R W;
  if (slabw) {
    const R kk = a.kap[dc][pw], ss = a.sig[dc][pw];
    const R fwn = (gs * in.us);
    o.fw = fwn;
    o.wfw = true;
    o.e = in.e + ((kk + ss) * fwn - (kk - ss) * in.fw);
    W = fwn;
  }
  else {
    o.e = (gs * in.us);
    o.fw = R(0);
    o.wfw = false;
    W = o.e;
  }
#pragma unroll
  for (int q = 0; q < NP; q++)
    o.pn[q] = a.pg1inv[q] * (in.p[q] * (R(2) - a.pw0d[q]) - a.pg1[q] * in.pp[q] + a.pw0[q] * (in.s[q] * W));
  return o;
}
template <typename R, int NP>
__device__ __forceinline__ void epole_store(const FusedArgs<R> &a, int dc, int i, const EPoleIn<R, NP> &in,
                                            const EPoleOut<R, NP> &o) {
  a.e[dc][i] = o.e;
  if (o.wfw) a.fw[0][dc][i] = o.fw;
#pragma unroll
  for (int q = 0; q < NP; q++)
    if (in.on[q]) {
      a.P[q][dc][i] = o.pn[q];
      a.PP[q][dc][i] = in.p[q];
    }
}

// NP: number of poles held in registers (0 none, 1 or 2), or -1 for any
// number, updated one component after the other
template <typename R, bool CND, int NP, bool FX, bool FY, bool FZ>
__device__ __forceinline__ void de3_point(const FusedArgs<R> &a, const int k[3]) {
  constexpr bool POLES = NP != 0;
  const int sx = a.s[0], sy = a.s[1];
  const int i = k[0] * sx + k[1] * sy + k[2];
  ShellFlags<R> F;
  band_flags<R, FX, FY, FZ>(a, k, F);
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
  bool hcx = CND && a.cnd[2][0] != nullptr, hcy = CND && a.cnd[2][1] != nullptr, hcz = CND && a.cnd[2][2] != nullptr;
  const unsigned am = (CND || POLES) ? seg_active(a, k) : 0u;
  // Dx (1,0,0): dsig = Y (shift 0), dsigu = Z (shift 0)
  if (hcx) hcx = F.s0[1] ? chunk_has(a.cond_chunks[2][0], F.r1[0], F.r0[1], F.r0[2]) : ((am >> (AM_DCOND + 0)) & 1u);
  // Dy (0,1,0): dsig = Z, dsigu = X
  if (hcy) hcy = F.s0[2] ? chunk_has(a.cond_chunks[2][1], F.r0[0], F.r1[1], F.r0[2]) : ((am >> (AM_DCOND + 1)) & 1u);
  // Dz (0,0,1): dsig = X, dsigu = Y
  if (hcz) hcz = F.s0[0] ? chunk_has(a.cond_chunks[2][2], F.r0[0], F.r0[1], F.r1[2]) : ((am >> (AM_DCOND + 2)) & 1u);
  const CurlIn<R> inx = curl_in(F.s0[1], F.s0[2], hcx, a.fu[2][0], a.fcnd[2][0], a.cnd[2][0], a.cndinv[2][0], i);
  const CurlIn<R> iny = curl_in(F.s0[2], F.s0[0], hcy, a.fu[2][1], a.fcnd[2][1], a.cnd[2][1], a.cndinv[2][1], i);
  const CurlIn<R> inz = curl_in(F.s0[0], F.s0[1], hcz, a.fu[2][2], a.fcnd[2][2], a.cnd[2][2], a.cndinv[2][2], i);
  // without poles, or with poles held in registers, the E operands too
  // (chi, E and f_w inside the slab along the component's own direction,
  // the poles' P, P_prev and sigma)
  EIn<R> ex, ey, ez;
  if constexpr (!POLES) {
    ex = e_in(a, 0, i, vx, F.s1[0]);
    ey = e_in(a, 1, i, vy, F.s1[1]);
    ez = e_in(a, 2, i, vz, F.s1[2]);
  }
  constexpr int NPR = NP > 0 ? NP : 1;
  EPoleIn<R, NPR> qx, qy, qz;
  if constexpr (NP > 0) {
    qx = epole_in<R, NP>(a, 0, i, vx, F.s1[0], am);
    qy = epole_in<R, NP>(a, 1, i, vy, F.s1[1], am);
    qz = epole_in<R, NP>(a, 2, i, vz, F.s1[2], am);
  }
  const CurlRes<R> cx = curl_general(dx, Xx, dtdx, dt2, F.s0[1], F.s0[2], hcx, a.sig[1], a.kap[1], a.siginv[1], p0y,
                                     a.sig[2], a.kap[2], a.siginv[2], p0z, inx);
  const CurlRes<R> cy = curl_general(dy, Xy, dtdx, dt2, F.s0[2], F.s0[0], hcy, a.sig[2], a.kap[2], a.siginv[2], p0z,
                                     a.sig[0], a.kap[0], a.siginv[0], p0x, iny);
  const CurlRes<R> cz = curl_general(dz, Xz, dtdx, dt2, F.s0[0], F.s0[1], hcz, a.sig[0], a.kap[0], a.siginv[0], p0x,
                                     a.sig[1], a.kap[1], a.siginv[1], p0y, inz);
  // E components share the D positions: f_w slab along their own direction at
  // shift 1.  Without poles all loads go first, then the stores; with poles
  // (four more arrays per pole and component) one component after the other
  // keeps the registers, and so the occupancy, in bounds.
  EShell<R> ox, oy, oz;
  if constexpr (NP > 0) {
    EPoleOut<R, NPR> rx, ry, rz;
    if (vx) rx = epole_from<R, NP>(a, 0, cx.f, F.s1[0], p1x, qx);
    if (vy) ry = epole_from<R, NP>(a, 1, cy.f, F.s1[1], p1y, qy);
    if (vz) rz = epole_from<R, NP>(a, 2, cz.f, F.s1[2], p1z, qz);
    if (vx) {
      a.d[0][i] = cx.f;
      if (cx.wfu) a.fu[2][0][i] = cx.fu;
      if (cx.wfc) a.fcnd[2][0][i] = cx.fc;
      epole_store<R, NP>(a, 0, i, qx, rx);
    }
    if (vy) {
      a.d[1][i] = cy.f;
      if (cy.wfu) a.fu[2][1][i] = cy.fu;
      if (cy.wfc) a.fcnd[2][1][i] = cy.fc;
      epole_store<R, NP>(a, 1, i, qy, ry);
    }
    if (vz) {
      a.d[2][i] = cz.f;
      if (cz.wfu) a.fu[2][2][i] = cz.fu;
      if (cz.wfc) a.fcnd[2][2][i] = cz.fc;
      epole_store<R, NP>(a, 2, i, qz, rz);
    }
    return;
  }
  if constexpr (POLES) {
    if (vx) {
      ox = e_general<R, POLES>(a, 0, i, cx.f, F.s1[0], p1x, am);
      a.d[0][i] = cx.f;
      if (cx.wfu) a.fu[2][0][i] = cx.fu;
      if (cx.wfc) a.fcnd[2][0][i] = cx.fc;
      e_store<R, POLES>(a, 0, i, ox, am);
    }
    if (vy) {
      oy = e_general<R, POLES>(a, 1, i, cy.f, F.s1[1], p1y, am);
      a.d[1][i] = cy.f;
      if (cy.wfu) a.fu[2][1][i] = cy.fu;
      if (cy.wfc) a.fcnd[2][1][i] = cy.fc;
      e_store<R, POLES>(a, 1, i, oy, am);
    }
    if (vz) {
      oz = e_general<R, POLES>(a, 2, i, cz.f, F.s1[2], p1z, am);
      a.d[2][i] = cz.f;
      if (cz.wfu) a.fu[2][2][i] = cz.fu;
      if (cz.wfc) a.fcnd[2][2][i] = cz.fc;
      e_store<R, POLES>(a, 2, i, oz, am);
    }
    return;
  }
  if (vx) ox = e_from(a, 0, cx.f, F.s1[0], p1x, ex);
  if (vy) oy = e_from(a, 1, cy.f, F.s1[1], p1y, ey);
  if (vz) oz = e_from(a, 2, cz.f, F.s1[2], p1z, ez);
  if (vx) {
    a.d[0][i] = cx.f;
    if (cx.wfu) a.fu[2][0][i] = cx.fu;
    if (cx.wfc) a.fcnd[2][0][i] = cx.fc;
    e_store<R, POLES>(a, 0, i, ox, am);
  }
  if (vy) {
    a.d[1][i] = cy.f;
    if (cy.wfu) a.fu[2][1][i] = cy.fu;
    if (cy.wfc) a.fcnd[2][1][i] = cy.fc;
    e_store<R, POLES>(a, 1, i, oy, am);
  }
  if (vz) {
    a.d[2][i] = cz.f;
    if (cz.wfu) a.fu[2][2][i] = cz.fu;
    if (cz.wfc) a.fcnd[2][2][i] = cz.fc;
    e_store<R, POLES>(a, 2, i, oz, am);
  }
}

// Off-diagonal inverse permittivity: E along d reads D - P of the other
// components at the four points around it, so the D/E half-step runs as two
// passes.  Pass 1: D (with f_u, f_cond) exactly as in de3_point, then
// f_minus_p = D - P (poles in list order) where the component has poles or
// integrated sources (src/update_eh.cpp:108-123).
template <typename R, bool CND, bool FX, bool FY, bool FZ>
__device__ __forceinline__ void d3_point(const FusedArgs<R> &a, const int k[3]) {
  const int sx = a.s[0], sy = a.s[1];
  const int i = k[0] * sx + k[1] * sy + k[2];
  ShellFlags<R> F;
  band_flags<R, FX, FY, FZ>(a, k, F);
  const bool vx = k[1] >= 1 && k[2] >= 1, vy = k[0] >= 1 && k[2] >= 1, vz = k[0] >= 1 && k[1] >= 1;
  const R *Hx = F.s0[0] ? a.h[0] : a.b[0];
  const R *Hy = F.s0[1] ? a.h[1] : a.b[1];
  const R *Hz = F.s0[2] ? a.h[2] : a.b[2];
  const int mx = k[0] >= 1 ? sx : 0, my = k[1] >= 1 ? sy : 0, mz = k[2] >= 1 ? 1 : 0;
  const R hx = Hx[i], hxy = Hx[i - my], hxz = Hx[i - mz];
  const R hy = Hy[i], hyx = Hy[i - mx], hyz = Hy[i - mz];
  const R hz = Hz[i], hzx = Hz[i - mx], hzy = Hz[i - my];
  const R dx = a.d[0][i], dy = a.d[1][i], dz = a.d[2][i];
  const R Xx = (hzy - hz) + hy - hyz;
  const R Xy = (hxz - hx) + hz - hzx;
  const R Xz = (hyx - hy) + hx - hxy;
  const R dtdx = a.dtdx, dt2 = a.dt2;
  const int p0x = 2 * k[0], p0y = 2 * k[1], p0z = 2 * k[2];
  bool hcx = CND && a.cnd[2][0] != nullptr, hcy = CND && a.cnd[2][1] != nullptr, hcz = CND && a.cnd[2][2] != nullptr;
  const unsigned am = seg_active(a, k);
  if (hcx) hcx = F.s0[1] ? chunk_has(a.cond_chunks[2][0], F.r1[0], F.r0[1], F.r0[2]) : ((am >> (AM_DCOND + 0)) & 1u);
  if (hcy) hcy = F.s0[2] ? chunk_has(a.cond_chunks[2][1], F.r0[0], F.r1[1], F.r0[2]) : ((am >> (AM_DCOND + 1)) & 1u);
  if (hcz) hcz = F.s0[0] ? chunk_has(a.cond_chunks[2][2], F.r0[0], F.r0[1], F.r1[2]) : ((am >> (AM_DCOND + 2)) & 1u);
  const CurlIn<R> inx = curl_in(F.s0[1], F.s0[2], hcx, a.fu[2][0], a.fcnd[2][0], a.cnd[2][0], a.cndinv[2][0], i);
  const CurlIn<R> iny = curl_in(F.s0[2], F.s0[0], hcy, a.fu[2][1], a.fcnd[2][1], a.cnd[2][1], a.cndinv[2][1], i);
  const CurlIn<R> inz = curl_in(F.s0[0], F.s0[1], hcz, a.fu[2][2], a.fcnd[2][2], a.cnd[2][2], a.cndinv[2][2], i);
  const CurlRes<R> c[3] = {
      curl_general(dx, Xx, dtdx, dt2, F.s0[1], F.s0[2], hcx, a.sig[1], a.kap[1], a.siginv[1], p0y, a.sig[2],
                   a.kap[2], a.siginv[2], p0z, inx),
      curl_general(dy, Xy, dtdx, dt2, F.s0[2], F.s0[0], hcy, a.sig[2], a.kap[2], a.siginv[2], p0z, a.sig[0],
                   a.kap[0], a.siginv[0], p0x, iny),
      curl_general(dz, Xz, dtdx, dt2, F.s0[0], F.s0[1], hcz, a.sig[0], a.kap[0], a.siginv[0], p0x, a.sig[1],
                   a.kap[1], a.siginv[1], p0y, inz)};
  const bool v[3] = {vx, vy, vz};
#pragma unroll
  for (int dc = 0; dc < 3; dc++) {
    if (!v[dc]) continue;
    a.d[dc][i] = c[dc].f;
    if (c[dc].wfu) a.fu[2][dc][i] = c[dc].fu;
    if (c[dc].wfc) a.fcnd[2][dc][i] = c[dc].fc;
    if (a.fmp[dc]) {
      R g = c[dc].f;
#pragma unroll
      for (int q = 0; q < MAX_POLES; q++)
        if (pole_on(a, am, q, dc)) g -= a.P[q][dc][i];
      a.fmp[dc][i] = g;
    }
  }
}

// Pass 2: E = chi_dd g + OFFDIAG terms (g = f_minus_p or D), f_w inside the
// slab along E's own direction, then the poles (src/step_generic.cpp:566-785,
// OFFDIAG :580-582).
template <typename R, bool POLES, bool FX, bool FY, bool FZ>
__device__ __forceinline__ void e3_point(const FusedArgs<R> &a, const int k[3]) {
  const int sx = a.s[0], sy = a.s[1];
  const int i = k[0] * sx + k[1] * sy + k[2];
  ShellFlags<R> F;
  band_flags<R, FX, FY, FZ>(a, k, F);
  const bool v[3] = {k[1] >= 1 && k[2] >= 1, k[0] >= 1 && k[2] >= 1, k[0] >= 1 && k[1] >= 1};
  const int pw[3] = {2 * k[0] + 1, 2 * k[1] + 1, 2 * k[2] + 1};
  const unsigned am = POLES ? seg_active(a, k) : 0u;
#pragma unroll
  for (int dc = 0; dc < 3; dc++) {
    if (!v[dc]) continue;
    const R *G = a.fmp[dc] ? a.fmp[dc] : a.d[dc];
    const R gs = G[i], us = a.chi[dc][i];
    R val = (gs * us);
    const int s = a.s[dc];
#pragma unroll
    for (int q = 0; q < 2; q++) {
      if (q >= a.noff[dc]) break;
      const int od = a.odir[dc][q], sxo = a.osx[dc][q];
      const R *g = a.fmp[od] ? a.fmp[od] : a.d[od];
      const R *u = a.chio[dc][q];
      val = val + R(0.25) * ((g[i] + g[i - sxo]) * u[i] + (g[i + s] + g[(i + s) - sxo]) * u[i + s]);
    }
    EShell<R> o;
    o.wfw = false;
    o.fw = R(0);
    R W;
    if (F.s1[dc]) {
      const R fwprev = a.fw[0][dc][i], kk = a.kap[dc][pw[dc]], ss = a.sig[dc][pw[dc]];
      o.fw = val;
      o.wfw = true;
      o.e = a.e[dc][i] + ((kk + ss) * val - (kk - ss) * fwprev);
      W = val;
    }
    else {
      o.e = val;
      W = o.e;
    }
    if (POLES) {
#pragma unroll
      for (int q = 0; q < MAX_POLES; q++)
        if (pole_on(a, am, q, dc)) {
          o.pc[q] = a.P[q][dc][i];
          o.pn[q] = a.pg1inv[q] * (o.pc[q] * (R(2) - a.pw0d[q]) - a.pg1[q] * a.PP[q][dc][i] +
                                   a.pw0[q] * (a.ps[q][dc][i] * W));
        }
    }
    e_store<R, POLES>(a, dc, i, o, am);
  }
}

template <typename R, bool CND, bool FX, bool FY, bool FZ>
__global__ void __launch_bounds__(256, 8) d3_band_kernel(const FusedArgs<R> a, const Band bd) {
  int k[3];
  if (band_coords(bd, k)) d3_point<R, CND, FX, FY, FZ>(a, k);
}

template <typename R, bool POLES, bool FX, bool FY, bool FZ>
__global__ void __launch_bounds__(256, 8) e3_band_kernel(const FusedArgs<R> a, const Band bd) {
  int k[3];
  if (band_coords(bd, k)) e3_point<R, POLES, FX, FY, FZ>(a, k);
}

// slab bands keep more operands in flight per point (every load issued
// before the branches): 40 registers there (64 in FP64), 32 in the rows
template <typename R, bool CND, bool FX, bool FY, bool FZ>
__global__ void __launch_bounds__(256, (FX || FY) ? (sizeof(R) == 8 ? 4 : 6) : 8)
    b3_band_kernel(const FusedArgs<R> a, const Band bd) {
  int k[3];
  if (band_coords(bd, k)) b3_point<R, CND, FX, FY, FZ>(a, k);
}

// true when every z point of this block's part of the band lies between the
// z slabs: both half-pixel positions of each point in the middle region, so
// the code without z PML gives the same arithmetic there (band_flags)
template <typename R> __device__ __forceinline__ bool z_interior_block(const FusedArgs<R> &a, const Band &bd) {
  const Span &s = bd.s[2];
  if (s.split < s.n) return false; // two runs: the general code
  const int t0 = (int)(blockIdx.x * blockDim.x);
  const int t1 = min(t0 + (int)blockDim.x, s.n) - 1;
  const bool lo = a.T[2][0] <= 0 || t0 + s.a0 >= a.T[2][0] + 1;
  const bool hi = a.T[2][1] <= 0 || t1 + s.a0 <= a.N[2] - a.T[2][1] - 1;
  return lo && hi;
}

// with poles in registers every operand of a point is loaded before any
// store: 64 registers (half occupancy, each thread keeps ~30 loads in flight).
// Without poles, rows that hold z slabs (FZ) run the code without z PML in
// their blocks between the slabs (block-uniform branch; 7 us per step on the
// 256^3 rows, measured slower with the pole kernels).
template <typename R, bool CND, int NP, bool FX, bool FY, bool FZ>
__global__ void __launch_bounds__(256, NP > 0 ? 4 : ((FX || FY) ? (sizeof(R) == 8 ? 4 : 6) : 8))
    de3_band_kernel(const FusedArgs<R> a, const Band bd) {
  int k[3];
  if (!band_coords(bd, k)) return;
  if constexpr (FZ && NP == 0) {
    if (z_interior_block(a, bd)) {
      de3_point<R, CND, NP, FX, FY, false>(a, k);
      return;
    }
  }
  de3_point<R, CND, NP, FX, FY, FZ>(a, k);
}

// The shell of a 3-D half-step in one launch: the z-interior x and y faces,
// their z edges and the x-y edges.  Each band keeps its own compile-time PML
// directions; a block of 32 x 8 threads works on one band (blocks numbered
// band after band, in each band z blocks fastest, then y, then x), so the
// shell has one launch and one tail instead of five.
struct ShellSet {
  Band b[5];    // x face z interior, y face z interior, x face z edges, y face z edges, x-y edges
  int gz[5];    // blocks along z (32 points each) of each band
  int gy[5];    // blocks along y (8 rows each)
  int first[6]; // first block of each band; first[5] is the total
};

// point of this thread in band q of the shell; false past the band's end
__device__ __forceinline__ bool shell_coords(const ShellSet &s, int &q, int k[3]) {
  const int blk = blockIdx.x;
  q = 0;
#pragma unroll
  for (int r = 1; r < 5; r++)
    q += blk >= s.first[r] ? 1 : 0;
  Band bd;
  int gz, gy, f0;
  switch (q) { // constant indices: the parameters stay in the constant bank
    case 0: bd = s.b[0], gz = s.gz[0], gy = s.gy[0], f0 = s.first[0]; break;
    case 1: bd = s.b[1], gz = s.gz[1], gy = s.gy[1], f0 = s.first[1]; break;
    case 2: bd = s.b[2], gz = s.gz[2], gy = s.gy[2], f0 = s.first[2]; break;
    case 3: bd = s.b[3], gz = s.gz[3], gy = s.gy[3], f0 = s.first[3]; break;
    default: bd = s.b[4], gz = s.gz[4], gy = s.gy[4], f0 = s.first[4]; break;
  }
  const int lb = blk - f0;
  const int t[3] = {lb / (gz * gy), (lb / gz) % gy * 8 + (int)threadIdx.y, lb % gz * 32 + (int)threadIdx.x};
  if (t[1] >= bd.s[1].n || t[2] >= bd.s[2].n) return false;
#pragma unroll
  for (int d = 0; d < 3; d++)
    k[d] = t[d] + (t[d] < bd.s[d].split ? bd.s[d].a0 : bd.s[d].a1);
  return true;
}

// the x-y edge band of a shell (band 4): this block's z points all lie
// between the z slabs (z_interior_block for the shell's block numbering)
template <typename R> __device__ __forceinline__ bool shell_z_interior(const FusedArgs<R> &a, const ShellSet &s) {
  const Span &z = s.b[4].s[2];
  if (z.split < z.n) return false;
  const int lb = (int)blockIdx.x - s.first[4];
  const int t0 = lb % s.gz[4] * 32, t1 = min(t0 + 32, z.n) - 1;
  return (a.T[2][0] <= 0 || t0 + z.a0 >= a.T[2][0] + 1) && (a.T[2][1] <= 0 || t1 + z.a0 <= a.N[2] - a.T[2][1] - 1);
}

template <typename R, bool CND, bool ZP>
__global__ void __launch_bounds__(256, sizeof(R) == 8 ? 4 : 6) b3_shell_kernel(const FusedArgs<R> a, const ShellSet s) {
  int q, k[3];
  if (!shell_coords(s, q, k)) return;
  switch (q) {
    case 0: b3_point<R, CND, true, false, false>(a, k); break;
    case 1: b3_point<R, CND, false, true, false>(a, k); break;
    case 2: b3_point<R, CND, true, false, ZP>(a, k); break;
    case 3: b3_point<R, CND, false, true, ZP>(a, k); break;
    default:
      if (ZP && shell_z_interior(a, s)) b3_point<R, CND, true, true, false>(a, k);
      else b3_point<R, CND, true, true, ZP>(a, k);
      break;
  }
}

template <typename R, bool CND, int NP, bool ZP>
__global__ void __launch_bounds__(256, NP > 0 ? 4 : (sizeof(R) == 8 ? 4 : 6))
    de3_shell_kernel(const FusedArgs<R> a, const ShellSet s) {
  int q, k[3];
  if (!shell_coords(s, q, k)) return;
  switch (q) {
    case 0: de3_point<R, CND, NP, true, false, false>(a, k); break;
    case 1: de3_point<R, CND, NP, false, true, false>(a, k); break;
    case 2: de3_point<R, CND, NP, true, false, ZP>(a, k); break;
    case 3: de3_point<R, CND, NP, false, true, ZP>(a, k); break;
    default:
      if (NP == 0 && ZP && shell_z_interior(a, s)) de3_point<R, CND, NP, true, true, false>(a, k);
      else de3_point<R, CND, NP, true, true, ZP>(a, k);
      break;
  }
}

} // namespace cuda_impl
} // namespace mfd
