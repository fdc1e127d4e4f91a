// Fused half-step kernels: one launch advances every component of one field
// type (B with its PML H copy, then D with E and the polarisations) over the
// whole cell.  Component wiring (which E/H component and stride enter each
// curl, Yee shifts, PML directions) is resolved at compile time from the grid
// dimension and the allocated-component mask, so each thread runs straight-line
// code; blocks that lie entirely in the interior chunk take a branch-free path
// with no PML loads at all.  Arithmetic per point is the same sequence as the
// generic kernels in mfd_cuda.cuh (reference: step_curl, step_update_EDHB,
// lorentzian update_P), so results are identical to them.
#pragma once

namespace mfd {
namespace cuda_impl {

template <int DIM> __host__ __device__ constexpr bool dpresent(int d) {
  return DIM == 3 || (DIM == 2 && d < 2) || (DIM == 1 && d == 2);
}
__host__ __device__ constexpr bool has_comp(int mask, int t, int d) { return (mask >> (3 * t + d)) & 1; }
// Yee shift of a component of type t, direction dc, along d
template <int DIM> __host__ __device__ constexpr int yshift(int t, int dc, int d) {
  return dpresent<DIM>(d) ? (((t == 0 || t == 2) && d == dc) || ((t == 1 || t == 3) && d != dc) ? 1 : 0) : 0;
}

template <typename R> struct FusedArgs {
  R *e[3], *d[3], *b[3], *h[3];
  R *fu[4][3];   // [type D=2 / B=3][dir] (index by type)
  R *fw[2][3];   // [type E=0 / H=1][dir]
  R *fcnd[4][3];
  const R *chi[3];
  const R *cnd[4][3], *cndinv[4][3];
  unsigned cond_chunks[4][3];
  int npoles;
  R *P[MAX_POLES][3], *PP[MAX_POLES][3];
  const R *ps[MAX_POLES][3];
  R pg1inv[MAX_POLES], pg1[MAX_POLES], pw0[MAX_POLES], pw0d[MAX_POLES];
  R dtdx, dt2;
  int N[3], T[3][2], pml[3];
  int s[3];
  const R *sig[3], *kap[3], *siginv[3]; // PML tables by half-pixel position
  bool fuse_h;   // update H in the PML slab right after B
  // off-diagonal inverse permittivity (3-D, two-pass D/E): f_minus_p of each
  // D component (null: D itself), the off-diagonal terms of each E component
  // (arrays, strides of their directions) in the reference's order
  R *fmp[3];
  const R *chio[3][2];
  int noff[3], odir[3][2], osx[3][2];
  // activity bits per run of 32 consecutive z points (row segment, aligned on
  // z = 0, 32, ...): bit 3q+d pole q has a nonzero sigma on E_d somewhere in
  // the segment, bit 12+d (15+d) D_d (B_d) has a nonzero conductivity there.
  // A pole with zero sigma keeps P = P_prev = 0 and a zero conductivity
  // leaves (1 - dt/2 sigma) f - dt curl and its condinv product unchanged, so
  // the 3-D band kernels skip those loads outside the f_cond branch.  Null:
  // everything active.
  const unsigned *amask;
  int mext1, mnseg;
  // nonzero: every segment of this launch has the activity bits am_all
  // (bit 31 set as the mark), so no word is loaded
  unsigned am_all;
  __device__ __forceinline__ R tbs(int d, int p) const { return sig[d][p]; }
  __device__ __forceinline__ R tbk(int d, int p) const { return kap[d][p]; }
  __device__ __forceinline__ R tbsi(int d, int p) const { return siginv[d][p]; }
};

template <typename R> __device__ __forceinline__ bool fslab(const FusedArgs<R> &a, int d, int pos) {
  return a.pml[d] && ((a.T[d][0] > 0 && pos <= 2 * a.T[d][0]) ||
                      (a.T[d][1] > 0 && pos > 2 * (a.N[d] - a.T[d][1])));
}
template <typename R> __device__ __forceinline__ int fregion(const FusedArgs<R> &a, int d, int pos) {
  if (a.T[d][0] > 0 && pos <= 2 * a.T[d][0]) return 0;
  if (a.T[d][1] > 0 && pos > 2 * (a.N[d] - a.T[d][1])) return 2;
  return 1;
}

template <typename R, int DIM, int T, int DC>
__device__ __forceinline__ bool comp_in_range(const FusedArgs<R> &a, const int k[3]) {
  bool ok = true;
#pragma unroll
  for (int d = 0; d < 3; d++)
    if (dpresent<DIM>(d)) {
      const int lo = yshift<DIM>(T, DC, d) ? 0 : 1;
      ok = ok && k[d] >= lo && k[d] <= a.N[d] - 1;
    }
  return ok;
}

// Curl update of component (T = D or B, direction DC) at point i: the new
// field value and the new auxiliaries (f_u, f_cond), nothing stored.
template <typename R> struct CurlOut {
  R f, fu, fc;
  bool wfu, wfc;
};

template <typename R, int DIM, int MASK, int T, int DC>
__device__ __forceinline__ CurlOut<R> curl_point(const FusedArgs<R> &a, const int k[3], int i,
                                                 bool interior) {
  constexpr int SRC = (T == 3) ? 0 : 1; // B <- E, D <- H
  constexpr int PD = (DC + 2) % 3, PDER = (DC + 1) % 3, MD = (DC + 1) % 3, MDER = (DC + 2) % 3;
  constexpr bool HP = dpresent<DIM>(PDER) && has_comp(MASK, SRC, PD);
  constexpr bool HM = dpresent<DIM>(MDER) && has_comp(MASK, SRC, MD);
  constexpr int G1D = HP ? PD : MD, G1DER = HP ? PDER : MDER;
  constexpr bool TWO = HP && HM;
  constexpr bool FLIP = !HP;
  CurlOut<R> o;
  o.wfu = o.wfc = false;
  R *F = (T == 3) ? a.b[DC] : a.d[DC];
  const R fold = F[i];
  o.fu = o.fc = R(0);
  if (!HP && !HM) { // component without curl terms (not instantiated in practice)
    o.f = fold;
    return o;
  }
  const int s1 = (T == 3) ? a.s[G1DER] : -a.s[G1DER];
  const int s2 = TWO ? ((T == 3) ? a.s[MDER] : -a.s[MDER]) : 0;
  const R *G1, *G2 = nullptr;
  if (T == 3) {
    G1 = a.e[G1D];
    if (TWO) G2 = a.e[MD];
  }
  else {
    // H is a separate array only inside the PML slab along its own direction
    G1 = (!interior && fslab(a, G1D, 2 * k[G1D])) ? a.h[G1D] : a.b[G1D];
    if (TWO) G2 = (!interior && fslab(a, MD, 2 * k[MD])) ? a.h[MD] : a.b[MD];
  }
  R X = G1[i + s1] - G1[i];
  if (TWO) X = X + G2[i] - G2[i + s2];
  const R dtdx = FLIP ? -a.dtdx : a.dtdx;
  const R *cnd = a.cnd[T][DC];
  const R one = R(1);
  if (interior) {
    o.f = cnd ? ((one - a.dt2 * cnd[i]) * fold - dtdx * X) * a.cndinv[T][DC][i] : fold - dtdx * X;
    return o;
  }
  constexpr int DS = (DC + 1) % 3, DU = (DC + 2) % 3;
  const int ps = yshift<DIM>(T, DC, DS) + 2 * k[DS];
  const int pu = yshift<DIM>(T, DC, DU) + 2 * k[DU];
  const bool sgm = dpresent<DIM>(DS) && fslab(a, DS, ps);
  const bool su = dpresent<DIM>(DU) && fslab(a, DU, pu);
  bool hc = cnd != nullptr;
  if (sgm && hc) {
    int r = fregion(a, 0, yshift<DIM>(T, DC, 0) + 2 * k[0]) * 9 +
            fregion(a, 1, yshift<DIM>(T, DC, 1) + 2 * k[1]) * 3 + fregion(a, 2, yshift<DIM>(T, DC, 2) + 2 * k[2]);
    hc = (a.cond_chunks[T][DC] >> r) & 1u;
  }
  if (!sgm) {
    if (!su) {
      o.f = hc ? ((one - a.dt2 * cnd[i]) * fold - dtdx * X) * a.cndinv[T][DC][i] : fold - dtdx * X;
      return o;
    }
    R fprev = a.fu[T][DC][i];
    R fun = hc ? ((one - a.dt2 * cnd[i]) * fprev - dtdx * X) * a.cndinv[T][DC][i] : fprev - dtdx * X;
    o.fu = fun;
    o.wfu = true;
    o.f = a.tbsi(DU, pu) * ((a.tbk(DU, pu) - a.tbs(DU, pu)) * fold + fun - fprev);
    return o;
  }
  const R ks = a.tbk(DS, ps) - a.tbs(DS, ps), si = a.tbsi(DS, ps);
  if (!su) {
    if (hc) {
      R fcp = a.fcnd[T][DC][i];
      R fcn = ((one - a.dt2 * cnd[i]) * fcp - dtdx * X) * a.cndinv[T][DC][i];
      o.fc = fcn;
      o.wfc = true;
      o.f = (ks * fold + (fcn - fcp)) * si;
    }
    else
      o.f = (ks * fold - dtdx * X) * si;
    return o;
  }
  R fprev = a.fu[T][DC][i];
  R fun;
  if (hc) {
    R fcp = a.fcnd[T][DC][i];
    R fcn = ((one - a.dt2 * cnd[i]) * fcp - dtdx * X) * a.cndinv[T][DC][i];
    o.fc = fcn;
    o.wfc = true;
    fun = (ks * fprev + (fcn - fcp)) * si;
  }
  else
    fun = (ks * fprev - dtdx * X) * si;
  o.fu = fun;
  o.wfu = true;
  o.f = a.tbsi(DU, pu) * ((a.tbk(DU, pu) - a.tbs(DU, pu)) * fold + fun - fprev);
  return o;
}

template <typename R, int T, int DC>
__device__ __forceinline__ void curl_store_aux(const FusedArgs<R> &a, int i, const CurlOut<R> &o) {
  if (o.wfu) a.fu[T][DC][i] = o.fu;
  if (o.wfc) a.fcnd[T][DC][i] = o.fc;
}

// ------------------------------------------------------------ B (+ H) kernel
// Results of one B component at one point: new B, its auxiliaries and, in the
// PML slab along its direction, the new H and f_w (update_eh for H,
// src/step_generic.cpp:692-698 with u == NULL).
template <typename R> struct BOut {
  CurlOut<R> c;
  bool act, wh;
  R h, fw;
};

template <typename R, int DIM, int MASK, int DC>
__device__ __forceinline__ void b_compute(const FusedArgs<R> &a, const int k[3], int i, bool interior,
                                          BOut<R> &o) {
  o.act = o.wh = false;
  if constexpr (has_comp(MASK, 3, DC)) {
    if (!interior && !comp_in_range<R, DIM, 3, DC>(a, k)) return;
    o.act = true;
    o.c = curl_point<R, DIM, MASK, 3, DC>(a, k, i, interior);
    if (a.fuse_h && !interior && dpresent<DIM>(DC)) {
      const int kw = 2 * k[DC];
      if (fslab(a, DC, kw)) {
        R fwprev = a.fw[1][DC][i], kapwkw = a.tbk(DC, kw), sigwkw = a.tbs(DC, kw);
        o.fw = o.c.f;
        o.h = a.h[DC][i] + ((kapwkw + sigwkw) * o.c.f - (kapwkw - sigwkw) * fwprev);
        o.wh = true;
      }
    }
  }
}

template <typename R, int DC>
__device__ __forceinline__ void b_store(const FusedArgs<R> &a, int i, const BOut<R> &o) {
  if (!o.act) return;
  curl_store_aux<R, 3, DC>(a, i, o.c);
  a.b[DC][i] = o.c.f;
  if (o.wh) {
    a.fw[1][DC][i] = o.fw;
    a.h[DC][i] = o.h;
  }
}

// Boxes of points covered by one launch (the interior box, or the PML and
// wall boxes around it); blocks are assigned to boxes in order.
struct BoxList {
  int n;
  int lo[7][3], ext[7][3];
  int blk0[8]; // first block of each box; blk0[n] = total
  int bx[7], by[7]; // blocks along the fast / mid axis of each box
};

// point of this thread; false if outside its box
template <int DIM> __device__ __forceinline__ bool box_coords(const BoxList &L, int k[3]) {
  int b = blockIdx.x, q = 0;
  while (q + 1 < L.n && b >= L.blk0[q + 1])
    q++;
  b -= L.blk0[q];
  const int FA = DIM == 2 ? 1 : 2, MA = DIM == 2 ? 0 : (DIM == 3 ? 1 : 0), SA = DIM == 3 ? 0 : (DIM == 2 ? 2 : 1);
  const int bfast = b % L.bx[q];
  b /= L.bx[q];
  const int bmid = b % L.by[q];
  const int bslow = b / L.by[q];
  const int tf = bfast * blockDim.x + threadIdx.x;
  const int tm = bmid * blockDim.y + threadIdx.y;
  if (tf >= L.ext[q][FA] || tm >= L.ext[q][MA]) return false;
  k[FA] = L.lo[q][FA] + tf;
  k[MA] = L.lo[q][MA] + tm;
  k[SA] = L.lo[q][SA] + bslow;
  return true;
}

template <typename R, int DIM, int MASK, bool INTERIOR>
__global__ void __launch_bounds__(256) fused_b_kernel(FusedArgs<R> a, BoxList L) {
  int k[3];
  if (!box_coords<DIM>(L, k)) return;
  const int i = k[0] * a.s[0] + k[1] * a.s[1] + k[2] * a.s[2];
  // all loads and arithmetic first, stores last (no store can then alias a
  // later load, so the loads of all components are in flight together)
  BOut<R> o0, o1, o2;
  b_compute<R, DIM, MASK, 0>(a, k, i, INTERIOR, o0);
  b_compute<R, DIM, MASK, 1>(a, k, i, INTERIOR, o1);
  b_compute<R, DIM, MASK, 2>(a, k, i, INTERIOR, o2);
  b_store<R, 0>(a, i, o0);
  b_store<R, 1>(a, i, o1);
  b_store<R, 2>(a, i, o2);
}

// --------------------------------------------------- D, E and poles kernel
template <typename R> struct DEOut {
  CurlOut<R> c;
  R d, e, fw;
  R p[MAX_POLES], pp[MAX_POLES];
};

// New D, E (f_w) and polarisations of component DC at point i, nothing stored
// except the D-curl auxiliaries.  srcA: integrated source terms subtracted from
// D - P (update_eh f_minus_p, src/update_eh.cpp:108-137).
template <typename R, int DIM, int MASK, int DC>
__device__ __forceinline__ void de_point(const FusedArgs<R> &a, const int k[3], int i, bool interior,
                                         int nsrc, const R *srcA, DEOut<R> &o) {
  o.c = curl_point<R, DIM, MASK, 2, DC>(a, k, i, interior);
  o.d = o.c.f;
  R gs = o.d;
#pragma unroll
  for (int q = 0; q < MAX_POLES; q++)
    if (q < a.npoles && a.P[q][DC]) gs -= a.P[q][DC][i];
  for (int j = 0; j < nsrc; j++)
    gs -= srcA[j];
  const R us = a.chi[DC][i];
  R W;
  const int kw = 2 * k[DC] + yshift<DIM>(0, DC, DC);
  if (!interior && dpresent<DIM>(DC) && fslab(a, DC, kw)) {
    R fwprev = a.fw[0][DC][i], kapwkw = a.tbk(DC, kw), sigwkw = a.tbs(DC, kw);
    R fwn = (gs * us);
    o.fw = fwn;
    o.e = a.e[DC][i] + ((kapwkw + sigwkw) * fwn - (kapwkw - sigwkw) * fwprev);
    W = fwn;
  }
  else {
    o.e = (gs * us);
    o.fw = R(0);
    W = o.e;
  }
#pragma unroll
  for (int q = 0; q < MAX_POLES; q++)
    if (q < a.npoles && a.P[q][DC]) {
      R pcur = a.P[q][DC][i];
      o.p[q] = a.pg1inv[q] * (pcur * (R(2) - a.pw0d[q]) - a.pg1[q] * a.PP[q][DC][i] + a.pw0[q] * (a.ps[q][DC][i] * W));
      o.pp[q] = pcur;
    }
}

template <typename R, int DIM, int DC>
__device__ __forceinline__ void de_store(const FusedArgs<R> &a, const int k[3], int i, bool interior,
                                         const DEOut<R> &o) {
  curl_store_aux<R, 2, DC>(a, i, o.c);
  a.d[DC][i] = o.d;
  a.e[DC][i] = o.e;
  const int kw = 2 * k[DC] + yshift<DIM>(0, DC, DC);
  if (!interior && dpresent<DIM>(DC) && fslab(a, DC, kw)) a.fw[0][DC][i] = o.fw;
#pragma unroll
  for (int q = 0; q < MAX_POLES; q++)
    if (q < a.npoles && a.P[q][DC]) {
      a.P[q][DC][i] = o.p[q];
      a.PP[q][DC][i] = o.pp[q];
    }
}

template <typename R, int DIM, int MASK, int DC>
__device__ __forceinline__ bool de_compute(const FusedArgs<R> &a, const int k[3], int i, bool interior,
                                           DEOut<R> &o) {
  if constexpr (has_comp(MASK, 2, DC)) {
    if (!interior && !comp_in_range<R, DIM, 2, DC>(a, k)) return false;
    de_point<R, DIM, MASK, DC>(a, k, i, interior, 0, (const R *)nullptr, o);
    return true;
  }
  return false;
}

template <typename R, int DIM, int MASK, bool INTERIOR>
__global__ void __launch_bounds__(256) fused_de_kernel(FusedArgs<R> a, BoxList L) {
  int k[3];
  if (!box_coords<DIM>(L, k)) return;
  const int i = k[0] * a.s[0] + k[1] * a.s[1] + k[2] * a.s[2];
  DEOut<R> o0, o1, o2;
  const bool a0 = de_compute<R, DIM, MASK, 0>(a, k, i, INTERIOR, o0);
  const bool a1 = de_compute<R, DIM, MASK, 1>(a, k, i, INTERIOR, o1);
  const bool a2 = de_compute<R, DIM, MASK, 2>(a, k, i, INTERIOR, o2);
  if (a0) de_store<R, DIM, 0>(a, k, i, INTERIOR, o0);
  if (a1) de_store<R, DIM, 1>(a, k, i, INTERIOR, o1);
  if (a2) de_store<R, DIM, 2>(a, k, i, INTERIOR, o2);
}

// Integrated E sources: the new D/E/P of each source point, computed from the
// state before the fused D/E kernel (pre) and written after it (post).
template <typename R, int DIM, int MASK>
__global__ void fused_src_pre_kernel(FusedArgs<R> a, const SrcPoint *pts, int n, int dc, DipoleVals dv,
                                     DEOut<R> *out) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const SrcPoint &sp = pts[j];
  R A[MAXS];
  for (int t = 0; t < sp.nterm; t++)
    A[t] = R(src_term(sp, t, dv));
  int k[3] = {sp.k[0], sp.k[1], sp.k[2]};
  // the general (non-interior) path gives identical values in the interior
  if (dc == 0) {
    if constexpr (has_comp(MASK, 2, 0)) de_point<R, DIM, MASK, 0>(a, k, (int)sp.i, false, sp.nterm, A, out[j]);
  }
  else if (dc == 1) {
    if constexpr (has_comp(MASK, 2, 1)) de_point<R, DIM, MASK, 1>(a, k, (int)sp.i, false, sp.nterm, A, out[j]);
  }
  else {
    if constexpr (has_comp(MASK, 2, 2)) de_point<R, DIM, MASK, 2>(a, k, (int)sp.i, false, sp.nterm, A, out[j]);
  }
}

template <typename R, int DIM, int MASK>
__global__ void fused_src_post_kernel(FusedArgs<R> a, const SrcPoint *pts, int n, int dc, const DEOut<R> *in) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const SrcPoint &sp = pts[j];
  int k[3] = {sp.k[0], sp.k[1], sp.k[2]};
  if (dc == 0) {
    if constexpr (has_comp(MASK, 2, 0)) de_store<R, DIM, 0>(a, k, (int)sp.i, false, in[j]);
  }
  else if (dc == 1) {
    if constexpr (has_comp(MASK, 2, 1)) de_store<R, DIM, 1>(a, k, (int)sp.i, false, in[j]);
  }
  else {
    if constexpr (has_comp(MASK, 2, 2)) de_store<R, DIM, 2>(a, k, (int)sp.i, false, in[j]);
  }
}

} // namespace cuda_impl
} // namespace mfd
