// FP32 quads on the z-interior x and y slab faces of the 3-D shell.  Each thread advances four consecutive z points with one 128-bit
// load or store per array.  A face of the shell holds PML arithmetic along x
// (or y) only: its flags, chunk regions and PML table entries are the same
// for the four points, so the arithmetic is that of b3_point for bands with
// no z flags, element by element, with the table entries and branch choices
// taken once per thread.  One-point threads on these faces issue about five
// times more instructions per byte than the quad B core (70% issue-active,
// the address unit half busy); quads cut the instructions per point (the
// 256^3 step: 0.3852 -> 0.3797 ms).  D/E faces go to quads only without
// poles: with two poles the quad kernel needs 190 registers and ran slower
// than the one-point bands, which then stay in the shell launch.  (A D/E
// quad core beside one-point z ends ran slower than whole one-point rows:
// 0.398 against 0.384 ms; so did the B z ends of the rows as quads with the
// quads that straddle a slab edge done point by point: 0.391 against 0.380.)
//
// The z neighbour of a quad (E one point up for B, H one point down for D)
// comes from the next (previous) lane by a warp shuffle when that lane holds
// the next (previous) quad of the same row; otherwise the lane loads it.
#pragma once

namespace mfd {
namespace cuda_impl {

// element-wise float4 arithmetic
__device__ __forceinline__ float4 operator+(float4 a, float4 b) {
  return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
__device__ __forceinline__ float4 operator-(float4 a, float4 b) {
  return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w);
}
__device__ __forceinline__ float4 operator*(float4 a, float4 b) {
  return make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w);
}
__device__ __forceinline__ float4 operator*(float s, float4 b) {
  return make_float4(s * b.x, s * b.y, s * b.z, s * b.w);
}
__device__ __forceinline__ float4 operator*(float4 a, float s) {
  return make_float4(a.x * s, a.y * s, a.z * s, a.w * s);
}
__device__ __forceinline__ float4 operator-(float s, float4 b) {
  return make_float4(s - b.x, s - b.y, s - b.z, s - b.w);
}
__device__ __forceinline__ float4 z4() { return make_float4(0.f, 0.f, 0.f, 0.f); }
__device__ __forceinline__ float4 q4ldc(bool c, const float *p, int i) { return c ? q4ld(p, i) : z4(); }

// step_curl branches (curl_general) on a quad; table entries per thread
struct QCurlIn {
  float4 fu, fc, cnd, cndinv;
};
struct QCurlRes {
  float4 f, fu, fc;
  bool wfu, wfc;
};
__device__ __forceinline__ QCurlIn q_curl_in(bool sg, bool su, bool hc, const float *fu, const float *fcnd,
                                             const float *cnd, const float *cndinv, int i) {
  QCurlIn v;
  v.fu = q4ldc(su, fu, i);
  v.fc = q4ldc(sg && hc, fcnd, i);
  v.cnd = q4ldc(hc, cnd, i);
  v.cndinv = q4ldc(hc, cndinv, i);
  return v;
}
__device__ __forceinline__ QCurlRes q_curl_general(float4 fold, float4 X, float dtdx, float dt2, bool sg, bool su,
                                                   bool hc, const float *sig_s, const float *kap_s,
                                                   const float *si_s, int ps, const float *sig_u,
                                                   const float *kap_u, const float *si_u, int pu,
                                                   const QCurlIn &v) {
  QCurlRes o;
  o.wfu = o.wfc = false;
  o.fu = o.fc = z4();
  const float one = 1.f;
  if (!sg) {
    if (!su) {
      o.f = hc ? ((one - dt2 * v.cnd) * fold - dtdx * X) * v.cndinv : fold - dtdx * X;
      return o;
    }
    const float4 fprev = v.fu;
    const float4 fun = hc ? ((one - dt2 * v.cnd) * fprev - dtdx * X) * v.cndinv : fprev - dtdx * X;
    o.fu = fun;
    o.wfu = true;
    o.f = si_u[pu] * ((kap_u[pu] - sig_u[pu]) * fold + fun - fprev);
    return o;
  }
  const float ks = kap_s[ps] - sig_s[ps], si = si_s[ps];
  if (!su) {
    if (hc) {
      const float4 fcp = v.fc;
      const float4 fcn = ((one - dt2 * v.cnd) * fcp - dtdx * X) * v.cndinv;
      o.fc = fcn;
      o.wfc = true;
      o.f = (ks * fold + (fcn - fcp)) * si;
    }
    else
      o.f = (ks * fold - dtdx * X) * si;
    return o;
  }
  const float4 fprev = v.fu;
  float4 fun;
  if (hc) {
    const float4 fcp = v.fc;
    const float4 fcn = ((one - dt2 * v.cnd) * fcp - dtdx * X) * v.cndinv;
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

// B on a quad of a z-interior face (b3_point with FZ = false)
template <bool CND, bool FX, bool FY>
__device__ __forceinline__ void b3q_face(const FusedArgs<float> &a, const int k[3], bool on, bool loadn) {
  const int sx = a.s[0], sy = a.s[1];
  const int i = k[0] * sx + k[1] * sy + k[2];
  ShellFlags<float> F;
  band_flags<float, FX, FY, false>(a, k, F);
  const bool vx = k[0] >= 1, vy = k[1] >= 1; // z >= 32: every z point is advanced
  const float *Ex = a.e[0], *Ey = a.e[1], *Ez = a.e[2];
  const float4 ex = q4ld(Ex, i), exy = q4ld(Ex, i + sy);
  const float4 ey = q4ld(Ey, i), eyx = q4ld(Ey, i + sx);
  const float4 ez = q4ld(Ez, i), ezx = q4ld(Ez, i + sx), ezy = q4ld(Ez, i + sy);
  float nx = __shfl_down_sync(0xffffffffu, ex.x, 1), ny = __shfl_down_sync(0xffffffffu, ey.x, 1);
  if (loadn) {
    nx = Ex[i + 4];
    ny = Ey[i + 4];
  }
  const float4 exz = make_float4(ex.y, ex.z, ex.w, nx), eyz = make_float4(ey.y, ey.z, ey.w, ny);
  const float4 bx = q4ld(a.b[0], i), by = q4ld(a.b[1], i), bz = q4ld(a.b[2], i);
  const float4 Xx = (ezy - ez) + ey - eyz;
  const float4 Xy = (exz - ex) + ez - ezx;
  const float4 Xz = (eyx - ey) + ex - exy;
  const float dtdx = a.dtdx, dt2 = a.dt2;
  const int p0x = 2 * k[0], p1x = p0x + 1, p0y = 2 * k[1], p1y = p0y + 1, p1z = 2 * k[2] + 1;
  bool hcx = CND && a.cnd[3][0] != nullptr, hcy = CND && a.cnd[3][1] != nullptr, hcz = CND && a.cnd[3][2] != nullptr;
  const unsigned am = CND ? seg_active(a, k) : 0u;
  if (hcx) hcx = F.s1[1] ? chunk_has(a.cond_chunks[3][0], F.r0[0], F.r1[1], F.r1[2]) : ((am >> (AM_BCOND + 0)) & 1u);
  if (hcy) hcy = F.s1[2] ? chunk_has(a.cond_chunks[3][1], F.r1[0], F.r0[1], F.r1[2]) : ((am >> (AM_BCOND + 1)) & 1u);
  if (hcz) hcz = F.s1[0] ? chunk_has(a.cond_chunks[3][2], F.r1[0], F.r1[1], F.r0[2]) : ((am >> (AM_BCOND + 2)) & 1u);
  const QCurlIn inx = q_curl_in(F.s1[1], F.s1[2], hcx, a.fu[3][0], a.fcnd[3][0], a.cnd[3][0], a.cndinv[3][0], i);
  const QCurlIn iny = q_curl_in(F.s1[2], F.s1[0], hcy, a.fu[3][1], a.fcnd[3][1], a.cnd[3][1], a.cndinv[3][1], i);
  const QCurlIn inz = q_curl_in(F.s1[0], F.s1[1], hcz, a.fu[3][2], a.fcnd[3][2], a.cnd[3][2], a.cndinv[3][2], i);
  const bool hx = a.fuse_h && F.s0[0] && vx, hy = a.fuse_h && F.s0[1] && vy;
  const float4 fwx0 = q4ldc(hx, a.fw[1][0], i), hx0 = q4ldc(hx, a.h[0], i);
  const float4 fwy0 = q4ldc(hy, a.fw[1][1], i), hy0 = q4ldc(hy, a.h[1], i);
  const QCurlRes cx = q_curl_general(bx, Xx, dtdx, dt2, F.s1[1], F.s1[2], hcx, a.sig[1], a.kap[1], a.siginv[1],
                                     p1y, a.sig[2], a.kap[2], a.siginv[2], p1z, inx);
  const QCurlRes cy = q_curl_general(by, Xy, dtdx, dt2, F.s1[2], F.s1[0], hcy, a.sig[2], a.kap[2], a.siginv[2],
                                     p1z, a.sig[0], a.kap[0], a.siginv[0], p1x, iny);
  const QCurlRes cz = q_curl_general(bz, Xz, dtdx, dt2, F.s1[0], F.s1[1], hcz, a.sig[0], a.kap[0], a.siginv[0],
                                     p1x, a.sig[1], a.kap[1], a.siginv[1], p1y, inz);
  if (!on) return;
  if (vx) {
    q4st(a.b[0], i, cx.f);
    if (cx.wfu) q4st(a.fu[3][0], i, cx.fu);
    if (cx.wfc) q4st(a.fcnd[3][0], i, cx.fc);
    if (hx) {
      const float kk = a.kap[0][p0x], ss = a.sig[0][p0x];
      q4st(a.fw[1][0], i, cx.f);
      q4st(a.h[0], i, hx0 + ((kk + ss) * cx.f - (kk - ss) * fwx0));
    }
  }
  if (vy) {
    q4st(a.b[1], i, cy.f);
    if (cy.wfu) q4st(a.fu[3][1], i, cy.fu);
    if (cy.wfc) q4st(a.fcnd[3][1], i, cy.fc);
    if (hy) {
      const float kk = a.kap[1][p0y], ss = a.sig[1][p0y];
      q4st(a.fw[1][1], i, cy.f);
      q4st(a.h[1], i, hy0 + ((kk + ss) * cy.f - (kk - ss) * fwy0));
    }
  }
  q4st(a.b[2], i, cz.f);
  if (cz.wfu) q4st(a.fu[3][2], i, cz.fu);
  if (cz.wfc) q4st(a.fcnd[3][2], i, cz.fc);
}

// D and E on a quad of a z-interior face without poles (de3_point with FZ =
// false, NP = 0): the curl operands and the E operands (chi; E and f_w in the
// component's own slab) all loaded before any store
struct QEIn {
  float4 us, fw, e;
};
__device__ __forceinline__ QEIn q_e_in(const FusedArgs<float> &a, int dc, int i, bool v, bool slabw) {
  QEIn o;
  o.us = q4ldc(v, a.chi[dc], i);
  o.fw = q4ldc(v && slabw, a.fw[0][dc], i);
  o.e = q4ldc(v && slabw, a.e[dc], i);
  return o;
}
// E = chi D (through f_w in the slab) and its stores (e_from, element by element)
__device__ __forceinline__ void q_e_update(const FusedArgs<float> &a, int dc, int i, float4 dn, bool slabw, int pw,
                                           const QEIn &in) {
  if (slabw) {
    const float kk = a.kap[dc][pw], ss = a.sig[dc][pw];
    const float4 fwn = (dn * in.us);
    q4st(a.fw[0][dc], i, fwn);
    q4st(a.e[dc], i, in.e + ((kk + ss) * fwn - (kk - ss) * in.fw));
  }
  else
    q4st(a.e[dc], i, (dn * in.us));
}

template <bool CND, bool FX, bool FY>
__device__ __forceinline__ void de3q_face(const FusedArgs<float> &a, const int k[3], bool on, bool loadp) {
  const int sx = a.s[0], sy = a.s[1];
  const int i = k[0] * sx + k[1] * sy + k[2];
  ShellFlags<float> F;
  band_flags<float, FX, FY, false>(a, k, F);
  const bool vx = k[1] >= 1, vy = k[0] >= 1, vz = k[0] >= 1 && k[1] >= 1; // z >= 32
  const float *Hx = F.s0[0] ? a.h[0] : a.b[0];
  const float *Hy = F.s0[1] ? a.h[1] : a.b[1];
  const float *Hz = a.b[2];
  const int mx = k[0] >= 1 ? sx : 0, my = k[1] >= 1 ? sy : 0;
  const float4 hx = q4ld(Hx, i), hxy = q4ld(Hx, i - my);
  const float4 hy = q4ld(Hy, i), hyx = q4ld(Hy, i - mx);
  const float4 hz = q4ld(Hz, i), hzx = q4ld(Hz, i - mx), hzy = q4ld(Hz, i - my);
  float px = __shfl_up_sync(0xffffffffu, hx.w, 1), py = __shfl_up_sync(0xffffffffu, hy.w, 1);
  if (loadp) {
    px = Hx[i - 1];
    py = Hy[i - 1];
  }
  const float4 hxz = make_float4(px, hx.x, hx.y, hx.z), hyz = make_float4(py, hy.x, hy.y, hy.z);
  const float4 dx = q4ld(a.d[0], i), dy = q4ld(a.d[1], i), dz = q4ld(a.d[2], i);
  const float4 Xx = (hzy - hz) + hy - hyz;
  const float4 Xy = (hxz - hx) + hz - hzx;
  const float4 Xz = (hyx - hy) + hx - hxy;
  const float dtdx = a.dtdx, dt2 = a.dt2;
  const int p0x = 2 * k[0], p1x = p0x + 1, p0y = 2 * k[1], p1y = p0y + 1, p0z = 2 * k[2];
  bool hcx = CND && a.cnd[2][0] != nullptr, hcy = CND && a.cnd[2][1] != nullptr, hcz = CND && a.cnd[2][2] != nullptr;
  const unsigned am = CND ? seg_active(a, k) : 0u;
  if (hcx) hcx = F.s0[1] ? chunk_has(a.cond_chunks[2][0], F.r1[0], F.r0[1], F.r0[2]) : ((am >> (AM_DCOND + 0)) & 1u);
  if (hcy) hcy = F.s0[2] ? chunk_has(a.cond_chunks[2][1], F.r0[0], F.r1[1], F.r0[2]) : ((am >> (AM_DCOND + 1)) & 1u);
  if (hcz) hcz = F.s0[0] ? chunk_has(a.cond_chunks[2][2], F.r0[0], F.r0[1], F.r1[2]) : ((am >> (AM_DCOND + 2)) & 1u);
  const QCurlIn inx = q_curl_in(F.s0[1], F.s0[2], hcx, a.fu[2][0], a.fcnd[2][0], a.cnd[2][0], a.cndinv[2][0], i);
  const QCurlIn iny = q_curl_in(F.s0[2], F.s0[0], hcy, a.fu[2][1], a.fcnd[2][1], a.cnd[2][1], a.cndinv[2][1], i);
  const QCurlIn inz = q_curl_in(F.s0[0], F.s0[1], hcz, a.fu[2][2], a.fcnd[2][2], a.cnd[2][2], a.cndinv[2][2], i);
  const QEIn qx = q_e_in(a, 0, i, vx, F.s1[0]);
  const QEIn qy = q_e_in(a, 1, i, vy, F.s1[1]);
  const QEIn qz = q_e_in(a, 2, i, vz, F.s1[2]);
  const QCurlRes cx = q_curl_general(dx, Xx, dtdx, dt2, F.s0[1], F.s0[2], hcx, a.sig[1], a.kap[1], a.siginv[1],
                                     p0y, a.sig[2], a.kap[2], a.siginv[2], p0z, inx);
  const QCurlRes cy = q_curl_general(dy, Xy, dtdx, dt2, F.s0[2], F.s0[0], hcy, a.sig[2], a.kap[2], a.siginv[2],
                                     p0z, a.sig[0], a.kap[0], a.siginv[0], p0x, iny);
  const QCurlRes cz = q_curl_general(dz, Xz, dtdx, dt2, F.s0[0], F.s0[1], hcz, a.sig[0], a.kap[0], a.siginv[0],
                                     p0x, a.sig[1], a.kap[1], a.siginv[1], p0y, inz);
  if (!on) return;
  if (vx) {
    q4st(a.d[0], i, cx.f);
    if (cx.wfu) q4st(a.fu[2][0], i, cx.fu);
    if (cx.wfc) q4st(a.fcnd[2][0], i, cx.fc);
    q_e_update(a, 0, i, cx.f, F.s1[0], p1x, qx);
  }
  if (vy) {
    q4st(a.d[1], i, cy.f);
    if (cy.wfu) q4st(a.fu[2][1], i, cy.fu);
    if (cy.wfc) q4st(a.fcnd[2][1], i, cy.fc);
    q_e_update(a, 1, i, cy.f, F.s1[1], p1y, qy);
  }
  if (vz) {
    q4st(a.d[2], i, cz.f);
    if (cz.wfu) q4st(a.fu[2][2], i, cz.fu);
    if (cz.wfc) q4st(a.fcnd[2][2], i, cz.fc);
    q_e_update(a, 2, i, cz.f, F.s1[2], 2 * k[2] + 1, qz);
  }
}

// the two z-interior faces as quads: blocks [0, nblk[0]) the x face, the rest
// the y face; in each face the quads of all rows are numbered row after row
struct QFaces {
  Band b[2];
  int nq[2];            // quads per row
  long long nquads[2];  // quads in the face
  int nblk[2];          // blocks of 256 quads
};

__device__ __forceinline__ void qface_coords(const QFaces &f, int &face, int k[3], bool &on, bool &first, bool &last) {
  face = (int)blockIdx.x >= f.nblk[0] ? 1 : 0;
  const long long t = (long long)((int)blockIdx.x - (face ? f.nblk[0] : 0)) * 256 + threadIdx.x;
  const long long nqs = face ? f.nquads[1] : f.nquads[0];
  on = t < nqs;
  const long long tq = on ? t : 0; // threads past the end take the first quad and store nothing
  const int nq = face ? f.nq[1] : f.nq[0];
  const Span s0 = face ? f.b[1].s[0] : f.b[0].s[0], s1 = face ? f.b[1].s[1] : f.b[0].s[1];
  const int z0 = face ? f.b[1].s[2].a0 : f.b[0].s[2].a0;
  const int q = (int)(tq % nq);
  const long long row = tq / nq;
  const int yi = (int)(row % s1.n), xi = (int)(row / s1.n);
  k[0] = xi + (xi < s0.split ? s0.a0 : s0.a1);
  k[1] = yi + (yi < s1.split ? s1.a0 : s1.a1);
  k[2] = z0 + 4 * q;
  first = q == 0;
  last = q == nq - 1;
}

template <bool CND>
__global__ void __launch_bounds__(256) b3q_faces_kernel(const FusedArgs<float> a, const QFaces f) {
  int face, k[3];
  bool on, first, last;
  qface_coords(f, face, k, on, first, last);
  const bool loadn = on && ((threadIdx.x & 31) == 31 || last);
  if (face == 0) b3q_face<CND, true, false>(a, k, on, loadn);
  else b3q_face<CND, false, true>(a, k, on, loadn);
}

template <bool CND>
__global__ void __launch_bounds__(256) de3q_faces_kernel(const FusedArgs<float> a, const QFaces f) {
  int face, k[3];
  bool on, first, last;
  qface_coords(f, face, k, on, first, last);
  const bool loadp = on && ((threadIdx.x & 31) == 0 || first);
  if (face == 0) de3q_face<CND, true, false>(a, k, on, loadp);
  else de3q_face<CND, false, true>(a, k, on, loadp);
}

} // namespace cuda_impl
} // namespace mfd
