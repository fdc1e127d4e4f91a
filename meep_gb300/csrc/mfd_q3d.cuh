// FP32 3-D core kernel on quads: each thread advances four consecutive
// points along the unit-stride axis z with one 128-bit load or store per
// array.  The core has no PML slab and no metal wall in any direction, so
// the update is the plain branch of step_curl (src/step_generic.cpp:94-113):
//   B -= dtdx * curl E     (forward differences)
// with the conductivity branch where the chunk has one.  The z neighbour one
// point up comes from the next lane by a warp shuffle; the last lane of the
// warp or of the row loads it.
//
// The B update reads 6 and writes 3 arrays per point; one-point threads
// leave it latency-bound well below the HBM rate, quads reach it.  The D/E
// update (12+ arrays per point) saturates HBM with one-point threads already
// and keeps them, as does the FP64 engine, which is bound by its FP64
// arithmetic rate.
#pragma once

namespace mfd {
namespace cuda_impl {

__device__ __forceinline__ float4 q4ld(const float *p, int i) { return *reinterpret_cast<const float4 *>(p + i); }
__device__ __forceinline__ void q4st(float *p, int i, float4 v) { *reinterpret_cast<float4 *>(p + i) = v; }

// x - c * X, element by element
__device__ __forceinline__ float4 q4axpy(float4 x, float c, float4 X) {
  return make_float4(x.x - c * X.x, x.y - c * X.y, x.z - c * X.z, x.w - c * X.w);
}
// (a - b) + c - d, element by element (the curl of step_curl)
__device__ __forceinline__ float4 q4curl(float4 a, float4 b, float4 c, float4 d) {
  return make_float4((a.x - b.x) + c.x - d.x, (a.y - b.y) + c.y - d.y, (a.z - b.z) + c.z - d.z,
                     (a.w - b.w) + c.w - d.w);
}
// conductivity branch: ((1 - dt2 * s) * f - dtdx * X) * inv
__device__ __forceinline__ float4 q4cond(float4 f, float4 X, float4 s, float4 inv, float dtdx, float dt2) {
  return make_float4(((1.f - dt2 * s.x) * f.x - dtdx * X.x) * inv.x, ((1.f - dt2 * s.y) * f.y - dtdx * X.y) * inv.y,
                     ((1.f - dt2 * s.z) * f.z - dtdx * X.z) * inv.z, ((1.f - dt2 * s.w) * f.w - dtdx * X.w) * inv.w);
}

template <bool CND>
__device__ __forceinline__ float4 q4step(const FusedArgs<float> &a, int t, int dc, int i, float4 f, float4 X) {
  if (CND && a.cnd[t][dc]) return q4cond(f, X, q4ld(a.cnd[t][dc], i), q4ld(a.cndinv[t][dc], i), a.dtdx, a.dt2);
  return q4axpy(f, a.dtdx, X);
}

// The core: x and y interior, z interior rounded inwards to whole quads
// (no PML slab and no metal wall in any direction).  The quads of all core
// rows are numbered row after row and a warp takes 32 consecutive ones, so
// no lane idles at the end of a row (a row holds 38 quads in the 384^2 x 192
// workload, 54 in the 256^3 one).
struct QCore {
  int lo[3]; // first point (lo[2] a multiple of 4, >= 4)
  int n[2];  // x and y extents
  int zend;  // one past the last z point (a multiple of 4)
  int nq;    // quads per row
  long long total; // quads in the core
};

template <bool CND>
__global__ void __launch_bounds__(256) b3q_core_kernel(const FusedArgs<float> a, const QCore b) {
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  // threads past the end take the first quad (they join the shuffle) and
  // store nothing
  const bool on = t < b.total;
  const long long tq = on ? t : 0;
  const int q = (int)(tq % b.nq);
  const long long row = tq / b.nq;
  const int k2 = b.lo[2] + 4 * q;
  const int k1 = b.lo[1] + (int)(row % b.n[1]);
  const int k0 = b.lo[0] + (int)(row / b.n[1]);
  const int i = k0 * a.s[0] + k1 * a.s[1] + k2;
  const int sx = a.s[0], sy = a.s[1];
  const float *__restrict__ Ex = a.e[0];
  const float *__restrict__ Ey = a.e[1];
  const float *__restrict__ Ez = a.e[2];
  const float4 ex = q4ld(Ex, i), exy = q4ld(Ex, i + sy);
  const float4 ey = q4ld(Ey, i), eyx = q4ld(Ey, i + sx);
  const float4 ez = q4ld(Ez, i), ezx = q4ld(Ez, i + sx), ezy = q4ld(Ez, i + sy);
  const float4 bx = q4ld(a.b[0], i), by = q4ld(a.b[1], i), bz = q4ld(a.b[2], i);
  // E one point up along z: the next lane's first element when that lane
  // holds the next quad of the same row; the last lane of the warp and the
  // last quad of a row load it (zend <= N: inside the row)
  float nx = __shfl_down_sync(0xffffffffu, ex.x, 1), ny = __shfl_down_sync(0xffffffffu, ey.x, 1);
  if (on && ((threadIdx.x & 31) == 31 || q == b.nq - 1)) {
    nx = Ex[i + 4];
    ny = Ey[i + 4];
  }
  const float4 exz = make_float4(ex.y, ex.z, ex.w, nx), eyz = make_float4(ey.y, ey.z, ey.w, ny);
  const float4 nbx = q4step<CND>(a, 3, 0, i, bx, q4curl(ezy, ez, ey, eyz));
  const float4 nby = q4step<CND>(a, 3, 1, i, by, q4curl(exz, ex, ez, ezx));
  const float4 nbz = q4step<CND>(a, 3, 2, i, bz, q4curl(eyx, ey, ex, exy));
  if (!on) return;
  q4st(a.b[0], i, nbx);
  q4st(a.b[1], i, nby);
  q4st(a.b[2], i, nbz);
}

} // namespace cuda_impl
} // namespace mfd
