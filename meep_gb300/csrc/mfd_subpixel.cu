// Subpixel averaging on the GPU (mfd_subpixel_rows, include/mfd.h).
//
// The reference averages pixel by pixel on the host
// (structure_chunk::set_chi1inv, src/anisotropic_averaging.cpp:211-324): per
// pixel a 50-point sphere quadrature for the interface normal, then grids of
// 10^d, 20^d, 40^d material evaluations until the means of eps and 1/eps
// settle -- about 7e4 evaluations for a pixel on an interface, summed in
// order.  The rows here are bit-identical to that routine (subpixel.hpp,
// which the CPU oracle runs as is); the work is split for the GPU:
//
//   normal kernel (one thread per pixel): the quadrature normal in IEEE
//     double over all objects; pixels that see one material (most of them)
//     are finished here, the others go to a work list with their gradient.
//   level kernel (warps of 32 listed pixels, one refinement level per
//     launch, the pixels that need the next level compacted into the next
//     list): per pixel the warp evaluates tiles of samples, then each lane
//     adds its own pixel's tile in sample order (details at the kernel);
//   mean kernel (one warp per pixel, for pixels meeting more than LMAXC
//     objects): the objects whose bounding box
//     meets the pixel are gathered in shared memory (list order kept); the
//     lanes evaluate the sample grid a tile at a time, deciding point-in-object
//     in FP32 with a margin of 1e-5 of the magnitudes involved (FP32 error is
//     ~1e-7 of them) and in exact double arithmetic when the FP32 value falls
//     inside the margin; lane 0 then adds the tile's eps and 1/eps to the
//     running sums in sample order, so the sums round exactly as the
//     reference's sequential loop does.  GB300 issues FP64 at a small fraction
//     of its FP32 rate, hence the FP32 filter.
//
// Compiled with --fmad=false: every double product and sum is rounded as in
// the reference's non-FMA x86-64 build.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <utility>
#include <vector>

#include "geom_eval.hpp"
#include "mfd.h"
#include "mfd_backend.hpp"
#include "subpixel.hpp"

namespace mfd {
namespace {

constexpr int MEAN_WARPS = 4;  // warps per block of the mean kernel
constexpr int MAXCAND = 32;    // culled objects per pixel kept in shared memory
constexpr int TABMAX = 128;    // per-axis sample coordinates tabulated (ms <= TABMAX)
constexpr int TILE = 128;      // samples per warp round
constexpr float MARGIN = 1e-5f;

struct DeviceChi {
  const mfd_object *objs;
  int nobj;
  double eps_default;
  __device__ double operator()(const double p[3]) const {
    const int q = mgb_geom::object_at(objs, nobj, p);
    return q < 0 ? eps_default : objs[q].eps;
  }
};

__device__ __forceinline__ void load_pixel(const double *lo, const double *hi, long long i, double l[3],
                                           double h[3]) {
  for (int d = 0; d < 3; d++) {
    l[d] = lo[3 * i + d];
    h[d] = hi[3 * i + d];
  }
}

// ---------------------------------------------------------------- phase 1
__global__ void __launch_bounds__(128)
    subpixel_normal_kernel(int dim, int cdir, long long npix, const double *lo, const double *hi, int maxeval,
                           const mgb_subpixel::SphereQuad *sq, DeviceChi chi, double *rows, double *grad,
                           int *work, int *nwork) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npix) return;
  double l[3], h[3];
  load_pixel(lo, hi, i, l, h);
  const bool act[3] = {dim >= 2, dim >= 2, dim != 2};
  double cen[3] = {0, 0, 0};
  for (int d = 0; d < 3; d++)
    if (act[d]) cen[d] = (h[d] + l[d]) * 0.5;
  if (maxeval) {
    double g[3];
    mgb_subpixel::normal_vector(dim, l, h, *sq, chi, g);
    double g2 = 0.0;
    for (int d = 0; d < 3; d++)
      if (act[d]) g2 += g[d] * g[d];
    if (sqrt(g2) >= 1e-8) {
      const int slot = atomicAdd(nwork, 1);
      work[slot] = (int)i;
      for (int d = 0; d < 3; d++)
        grad[3 * i + d] = g[d];
      return;
    }
  }
  rows[3 * i] = rows[3 * i + 1] = rows[3 * i + 2] = 0.0;
  rows[3 * i + cdir] = 1 / chi(cen);
}

// ---------------------------------------------------------------- phase 2
struct Cand {
  int obj, kind;
  float a[3];  // float(0 or lo - center): sample offset origin relative to the object
  float ax[3]; // cylinder axis
  float hs[3]; // block half sizes
  float r2, hh;
};

struct WarpShared {
  Cand cand[MAXCAND];
  double eps[MAXCAND + 1], inv[MAXCAND + 1];
  double tab[3][TABMAX];
  float tabf[3][TABMAX];
  double te[TILE], ti[TILE];
};

// +1 inside, -1 outside, 0 too close to the surface to decide in FP32
__device__ __forceinline__ int test32(const Cand &c, const float t[3]) {
  float d[3], m[3];
  for (int q = 0; q < 3; q++) {
    d[q] = c.a[q] + t[q];
    m[q] = fabsf(c.a[q]) + fabsf(t[q]);
  }
  if (c.kind == 0) {
    bool undecided = false;
    for (int q = 0; q < 3; q++) {
      const float v = fabsf(d[q]) - c.hs[q], mg = MARGIN * (m[q] + c.hs[q]);
      if (v > mg) return -1;
      if (v >= -mg) undecided = true;
    }
    return undecided ? 0 : 1;
  }
  if (c.kind == 1) {
    const float s = d[0] * d[0] + d[1] * d[1] + d[2] * d[2] - c.r2;
    const float mg = MARGIN * (m[0] * m[0] + m[1] * m[1] + m[2] * m[2] + c.r2);
    return s > mg ? -1 : (s < -mg ? 1 : 0);
  }
  const float hp = d[0] * c.ax[0] + d[1] * c.ax[1] + d[2] * c.ax[2];
  const float mh = m[0] * fabsf(c.ax[0]) + m[1] * fabsf(c.ax[1]) + m[2] * fabsf(c.ax[2]);
  const float v1 = fabsf(hp) - c.hh, mg1 = MARGIN * (mh + c.hh);
  if (v1 > mg1) return -1;
  float q2 = 0.f, mq = 0.f;
  for (int q = 0; q < 3; q++) {
    const float e = d[q] - hp * c.ax[q], me = m[q] + mh * fabsf(c.ax[q]);
    q2 += e * e;
    mq += me * me;
  }
  const float v2 = q2 - c.r2, mg2 = MARGIN * (mq + c.r2);
  if (v2 > mg2) return -1;
  return (v1 < -mg1 && v2 < -mg2) ? 1 : 0;
}

// conservative: false only if no point of [l, h] can be inside the object
__device__ __forceinline__ bool box_meets(const mfd_object &o, const double l[3], const double h[3],
                                          const bool act[3]) {
  for (int d = 0; d < 3; d++) {
    double ext;
    if (o.kind == 0) ext = 0.5 * o.size[d];
    else if (o.kind == 1) ext = o.radius;
    else ext = fabs(o.axis[d]) * 0.5 * o.height + o.radius;
    const double lo = act[d] ? l[d] : 0.0, hi = act[d] ? h[d] : 0.0;
    const double slack = 1e-9 * (1.0 + fabs(o.center[d]) + fabs(ext) + fabs(lo) + fabs(hi));
    if (hi < o.center[d] - ext - slack || lo > o.center[d] + ext + slack) return false;
  }
  return true;
}

__global__ void __launch_bounds__(32 * MEAN_WARPS)
    subpixel_mean_kernel(int dim, int cdir, const double *lo, const double *hi, double tol, int maxeval,
                         DeviceChi chi, const double *grad, const int *work, const int *nwork, double *rows) {
  __shared__ WarpShared sh_all[MEAN_WARPS];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  WarpShared &S = sh_all[wib];
  const int nw = *nwork;
  const bool act[3] = {dim >= 2, dim >= 2, dim != 2};
  for (int w = blockIdx.x * MEAN_WARPS + wib; w < nw; w += gridDim.x * MEAN_WARPS) {
    const long long pix = work[w];
    double l[3], h[3];
    load_pixel(lo, hi, pix, l, h);
    double cen[3] = {0, 0, 0}, ext[3] = {0, 0, 0}, org[3] = {0, 0, 0};
    for (int d = 0; d < 3; d++)
      if (act[d]) {
        cen[d] = (h[d] + l[d]) * 0.5;
        ext[d] = h[d] - l[d];
        org[d] = l[d];
      }
    // objects meeting the pixel, in list order (ordered compaction by ballot)
    int ncand = 0;
    bool overflow = false;
    for (int base = 0; base < chi.nobj; base += 32) {
      const int q = base + lane;
      const bool hit = q < chi.nobj && box_meets(chi.objs[q], l, h, act);
      const unsigned mask = __ballot_sync(0xffffffffu, hit);
      const int pos = ncand + __popc(mask & ((1u << lane) - 1u));
      if (hit && pos < MAXCAND) {
        const mfd_object &o = chi.objs[q];
        Cand &c = S.cand[pos];
        c.obj = q;
        c.kind = o.kind;
        for (int d = 0; d < 3; d++) {
          c.a[d] = (float)(org[d] - o.center[d]);
          c.ax[d] = (float)o.axis[d];
          c.hs[d] = (float)(0.5 * o.size[d]);
        }
        c.r2 = (float)(o.radius * o.radius);
        c.hh = (float)(0.5 * o.height);
        S.eps[pos] = o.eps;
        S.inv[pos] = 1 / o.eps;
      }
      ncand += __popc(mask);
    }
    if (ncand > MAXCAND) overflow = true;
    if (!overflow && lane == 0) {
      S.eps[ncand] = chi.eps_default;
      S.inv[ncand] = 1 / chi.eps_default;
    }
    __syncwarp();

    double meps = 1, minveps = 1, old_meps = 0, old_minveps = 0;
    int ms = 10, iter = 0;
    int state = 0; // 0 running, 1 done (means final), 2 trivial (negative eps)
    while (state == 0) {
      int go = 0;
      if (lane == 0)
        go = fabs(meps - old_meps) > tol * fabs(old_meps) && fabs(minveps - old_minveps) > tol * fabs(old_minveps);
      go = __shfl_sync(0xffffffffu, go, 0);
      if (!go) break;
      old_meps = meps;
      old_minveps = minveps;
      meps = minveps = 0;
      const int n2 = dim >= 2 ? ms : 1, n3 = dim >= 3 ? ms : 1;
      const int cnt = ms * n2 * n3;
      const bool fast = !overflow && ms <= TABMAX;
      if (fast) {
        // sample coordinates along each axis: lo + i * ext / ms, as in the
        // reference; axes absent from the grid are 0
        for (int d = 0; d < 3; d++) {
          const int nd = (dim == 1 && d < 2) || (dim == 2 && d == 2) ? 1 : ms;
          for (int i = lane; i < nd; i += 32) {
            const double t = act[d] ? i * ext[d] / ms : 0.0;
            S.tab[d][i] = act[d] ? l[d] + t : 0.0;
            S.tabf[d][i] = (float)t;
          }
        }
        __syncwarp();
      }
      int negative = 0;
      for (int base = 0; base < cnt; base += TILE) {
        const int nt = min(TILE, cnt - base);
        for (int s = lane; s < nt; s += 32) {
          const int idx = base + s;
          int ix, jy, kz;
          if (dim == 1) {
            ix = idx;
            jy = kz = 0;
          }
          else {
            ix = idx % ms;
            jy = (idx / ms) % n2;
            kz = idx / (ms * n2);
          }
          // (x, y, z) indices into the per-axis tables: 1-D samples run along z
          const int ti[3] = {dim == 1 ? 0 : ix, dim == 1 ? 0 : jy, dim == 1 ? ix : (dim == 3 ? kz : 0)};
          double ep, iv;
          if (fast) {
            const double p[3] = {S.tab[0][ti[0]], S.tab[1][ti[1]], S.tab[2][ti[2]]};
            const float t[3] = {S.tabf[0][ti[0]], S.tabf[1][ti[1]], S.tabf[2][ti[2]]};
            int hitc = ncand;
            for (int c = ncand - 1; c >= 0; c--) {
              int r = test32(S.cand[c], t);
              if (r == 0) r = mgb_geom::contains(chi.objs[S.cand[c].obj], p) ? 1 : -1;
              if (r > 0) {
                hitc = c;
                break;
              }
            }
            ep = S.eps[hitc];
            iv = S.inv[hitc];
          }
          else {
            double p[3] = {0, 0, 0};
            if (dim == 1) p[2] = l[2] + ix * ext[2] / ms;
            else {
              p[0] = l[0] + ix * ext[0] / ms;
              p[1] = l[1] + jy * ext[1] / ms;
              if (dim == 3) p[2] = l[2] + kz * ext[2] / ms;
            }
            ep = chi(p);
            iv = 1 / ep;
          }
          if (ep < 0) negative = 1;
          S.te[s] = ep;
          S.ti[s] = iv;
        }
        __syncwarp();
        if (lane == 0)
          for (int s = 0; s < nt; s++) {
            meps += S.te[s];
            minveps += S.ti[s];
          }
        __syncwarp();
      }
      negative = __any_sync(0xffffffffu, negative);
      if (negative) {
        state = dim != 1 ? 2 : 1;
        if (dim == 1 && lane == 0) {
          meps = chi(cen);
          minveps = 1 / meps;
        }
        break;
      }
      if (lane == 0) {
        meps /= cnt;
        minveps /= cnt;
      }
      ms *= 2;
      if (maxeval && (iter += (dim == 3 ? ms * ms * ms : ms * ms)) >= maxeval) break;
    }
    if (lane == 0) {
      double *row = rows + 3 * pix;
      if (state == 2) {
        row[0] = row[1] = row[2] = 0.0;
        row[cdir] = 1 / chi(cen);
      }
      else {
        double g[3], g2 = 0.0;
        for (int d = 0; d < 3; d++) {
          g[d] = grad[3 * pix + d];
          if (act[d]) g2 += g[d] * g[d];
        }
        const double inv = 1.0 / sqrt(g2);
        double n[3] = {0, 0, 0};
        for (int d = 0; d < 3; d++)
          if (act[d]) n[d] = g[d] * inv;
        for (int q = 0; q < 3; ++q)
          row[q] = n[cdir] * n[q] * (minveps - 1 / meps);
        row[cdir] += 1 / meps;
      }
    }
    __syncwarp();
  }
}

// ------------------------------------------------- phase 2, level by level
// The per-pixel-warp kernel above adds every sample on lane 0, and GB300
// issues a one-lane FP64 add at the cost of a full warp instruction.  Here a
// warp takes 32 listed pixels at one refinement level (the same ms for the
// whole list): for each pixel the warp evaluates a tile of samples (one per
// lane, FP32 filter, exact FP64 test near surfaces), then every lane adds its
// own pixel's tile in sample order -- 32 in-order sums per FP64 instruction.
// Pixels that need the next level are compacted into the next list, so the
// warps stay full.  A pixel meeting more than LMAXC objects' boxes goes to the
// per-pixel-warp kernel instead.
constexpr int LV_WARPS = 2; // warps per block
constexpr int LMAXC = 6;    // objects per pixel
constexpr int LTILE = 128;  // samples per pixel per round

constexpr int LQMAX = 512; // samples queued for the exact test per round

struct LvShared {
  Cand cand[32][LMAXC];
  double eps[32][LMAXC + 1], inv[32][LMAXC + 1];
  double lo[32][3], ext[32][3];
  unsigned char res[32][LTILE];
  unsigned short q[LQMAX]; // (pixel << 8) | sample of the round
  int nc[32], neg[32], nq;
};

// the material slot of sample si of pixel j in this round: FP32 tests in
// list order from the last object; `exact` settles undecided ones in double
// (false: return -1 at the first undecided object instead)
__device__ __forceinline__ int sample_slot(const LvShared &S, const DeviceChi &chi, int dim, const bool act[3],
                                           int j, const int ti[3], const float t[3], int ms, bool exact) {
  const int nc = S.nc[j];
  for (int c = nc - 1; c >= 0; c--) {
    int r = test32(S.cand[j][c], t);
    if (r == 0) {
      if (!exact) return -1;
      // lo + i * ext / ms, as in the reference
      double p[3];
      for (int d = 0; d < 3; d++)
        p[d] = act[d] ? S.lo[j][d] + ti[d] * S.ext[j][d] / ms : 0.0;
      r = mgb_geom::contains(chi.objs[S.cand[j][c].obj], p) ? 1 : -1;
    }
    if (r > 0) return c;
  }
  (void)dim;
  return nc;
}

// the averaged row from the normal (gradient) and the means
__device__ __forceinline__ void row_from_means(int cdir, const bool act[3], const double *g3, double meps,
                                               double minveps, double *row) {
  double g[3], g2 = 0.0;
  for (int d = 0; d < 3; d++) {
    g[d] = g3[d];
    if (act[d]) g2 += g[d] * g[d];
  }
  const double inv = 1.0 / sqrt(g2);
  double n[3] = {0, 0, 0};
  for (int d = 0; d < 3; d++)
    if (act[d]) n[d] = g[d] * inv;
  for (int q = 0; q < 3; ++q)
    row[q] = n[cdir] * n[q] * (minveps - 1 / meps);
  row[cdir] += 1 / meps;
}

// means (meps, minveps) carried from one level to the next, per pixel
struct LvState {
  double meps, minveps;
};

__global__ void __launch_bounds__(32 * LV_WARPS, 6)
    subpixel_level_kernel(int dim, int cdir, const double *lo, const double *hi, double tol, int ms, int first,
                          int stop, DeviceChi chi, const double *grad, const int *win, int nin, LvState *st,
                          int *wnext, int *nnext, int *wover, int *nover, double *rows) {
  __shared__ LvShared sh_all[LV_WARPS];
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  LvShared &S = sh_all[wib];
  const bool act[3] = {dim >= 2, dim >= 2, dim != 2};
  const int n2 = dim >= 2 ? ms : 1, n3 = dim >= 3 ? ms : 1, cnt = ms * n2 * n3;
  for (int w0 = (blockIdx.x * LV_WARPS + wib) * 32; w0 < nin; w0 += gridDim.x * LV_WARPS * 32) {
    const int item = w0 + lane;
    const bool mine = item < nin;
    const int pix = mine ? win[item] : 0;
    double l[3] = {0, 0, 0}, h[3] = {0, 0, 0};
    if (mine) load_pixel(lo, hi, pix, l, h);
    double cen[3] = {0, 0, 0};
    for (int d = 0; d < 3; d++)
      if (act[d]) cen[d] = (h[d] + l[d]) * 0.5;
    // the objects meeting each pixel of the warp, in list order
    for (int j = 0; j < 32; j++) {
      const int jmine = __shfl_sync(full, (int)mine, j);
      double lj[3], hj[3];
      for (int d = 0; d < 3; d++) {
        lj[d] = __shfl_sync(full, l[d], j);
        hj[d] = __shfl_sync(full, h[d], j);
      }
      if (!jmine) {
        if (lane == 0) S.nc[j] = 0;
        continue;
      }
      int nc = 0;
      for (int base = 0; base < chi.nobj; base += 32) {
        const int q = base + lane;
        const bool hit = q < chi.nobj && box_meets(chi.objs[q], lj, hj, act);
        const unsigned mask = __ballot_sync(full, hit);
        const int pos = nc + __popc(mask & ((1u << lane) - 1u));
        if (hit && pos < LMAXC) {
          const mfd_object &o = chi.objs[q];
          Cand &c = S.cand[j][pos];
          c.obj = q;
          c.kind = o.kind;
          for (int d = 0; d < 3; d++) {
            c.a[d] = (float)((act[d] ? lj[d] : 0.0) - o.center[d]);
            c.ax[d] = (float)o.axis[d];
            c.hs[d] = (float)(0.5 * o.size[d]);
          }
          c.r2 = (float)(o.radius * o.radius);
          c.hh = (float)(0.5 * o.height);
          S.eps[j][pos] = o.eps;
          S.inv[j][pos] = 1 / o.eps;
        }
        nc += __popc(mask);
      }
      if (lane < 3) {
        S.lo[j][lane] = act[lane] ? lj[lane] : 0.0;
        S.ext[j][lane] = act[lane] ? hj[lane] - lj[lane] : 0.0;
      }
      if (lane == 0) {
        S.nc[j] = nc;
        if (nc <= LMAXC) {
          S.eps[j][nc] = chi.eps_default;
          S.inv[j][nc] = 1 / chi.eps_default;
        }
      }
    }
    S.neg[lane] = 0;
    __syncwarp();
    const bool run = mine && S.nc[lane] <= LMAXC;
    if (mine && !run && first) wover[atomicAdd(nover, 1)] = pix;
    double old_meps = 1, old_minveps = 1;
    if (run && !first) {
      old_meps = st[pix].meps;
      old_minveps = st[pix].minveps;
    }
    double sm = 0, smi = 0;
    for (int base = 0; base < cnt; base += LTILE) {
      const int nt = min(LTILE, cnt - base);
      if (lane == 0) S.nq = 0;
      __syncwarp();
      for (int j = 0; j < 32; j++) {
        const int jrun = __shfl_sync(full, (int)run, j);
        if (!jrun) continue;
        // sample spacing in FP32 for the filter (ext / ms to ~1e-7: far inside
        // the filter's margin)
        const float stf[3] = {(float)(S.ext[j][0] / ms), (float)(S.ext[j][1] / ms), (float)(S.ext[j][2] / ms)};
        // this lane's samples si = lane + 32 m: grid indices carried forward
        // by 32 at a time
        int ix, jy, kz;
        {
          const int idx = base + lane;
          if (dim == 1) {
            ix = idx;
            jy = kz = 0;
          }
          else {
            ix = idx % ms;
            jy = (idx / ms) % n2;
            kz = idx / (ms * n2);
          }
        }
#pragma unroll 4
        for (int si = lane; si < nt; si += 32) {
          // per-axis sample index: 1-D samples run along z
          const int ti[3] = {dim == 1 ? 0 : ix, dim == 1 ? 0 : jy, dim == 1 ? ix : (dim == 3 ? kz : 0)};
          float t[3];
          for (int d = 0; d < 3; d++)
            t[d] = act[d] ? (float)ti[d] * stf[d] : 0.f;
          int slot = sample_slot(S, chi, dim, act, j, ti, t, ms, false);
          if (slot < 0) {
            // too close to a surface for FP32: queued for the exact test
            const int qn = atomicAdd(&S.nq, 1);
            if (qn < LQMAX) S.q[qn] = (unsigned short)((j << 8) | si);
            else slot = sample_slot(S, chi, dim, act, j, ti, t, ms, true);
          }
          if (slot >= 0) {
            S.res[j][si] = (unsigned char)slot;
            if (S.eps[j][slot] < 0) S.neg[j] = 1;
          }
          if (dim == 1)
            ix += 32;
          else {
            ix += 32;
            while (ix >= ms) {
              ix -= ms;
              if (++jy >= n2) {
                jy = 0;
                kz++;
              }
            }
          }
        }
      }
      __syncwarp();
      // the queued samples of all pixels of the round, with every lane busy
      const int nq = min(S.nq, LQMAX);
      for (int e = lane; e < nq; e += 32) {
        const int j = S.q[e] >> 8, si = S.q[e] & 0xff, idx = base + si;
        int ti[3] = {0, 0, 0};
        if (dim == 1) ti[2] = idx;
        else {
          ti[0] = idx % ms;
          ti[1] = (idx / ms) % n2;
          if (dim == 3) ti[2] = idx / (ms * n2);
        }
        float t[3];
        for (int d = 0; d < 3; d++)
          t[d] = act[d] ? (float)ti[d] * (float)(S.ext[j][d] / ms) : 0.f;
        const int slot = sample_slot(S, chi, dim, act, j, ti, t, ms, true);
        S.res[j][si] = (unsigned char)slot;
        if (S.eps[j][slot] < 0) S.neg[j] = 1;
      }
      __syncwarp();
      if (run)
        for (int q = 0; q < nt; q++) {
          const int c = S.res[lane][q];
          sm += S.eps[lane][c];
          smi += S.inv[lane][c];
        }
      __syncwarp();
    }
    if (run) {
      double *row = rows + 3 * pix;
      double meps = sm, minveps = smi;
      bool done;
      if (S.neg[lane]) {
        done = true;
        if (dim != 1) {
          row[0] = row[1] = row[2] = 0.0;
          row[cdir] = 1 / chi(cen);
        }
        else {
          meps = chi(cen);
          minveps = 1 / meps;
          row_from_means(cdir, act, grad + 3 * pix, meps, minveps, row);
        }
      }
      else {
        meps /= cnt;
        minveps /= cnt;
        done = stop || !(fabs(meps - old_meps) > tol * fabs(old_meps) &&
                         fabs(minveps - old_minveps) > tol * fabs(old_minveps));
        if (done) row_from_means(cdir, act, grad + 3 * pix, meps, minveps, row);
      }
      if (!done) {
        st[pix].meps = meps;
        st[pix].minveps = minveps;
        wnext[atomicAdd(nnext, 1)] = pix;
      }
    }
    __syncwarp();
  }
}

void check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw Error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

// device buffers freed on every exit path
struct DeviceBuffers {
  std::vector<void *> ptrs;
  template <class T> T *alloc(size_t n) {
    void *p = nullptr;
    check(cudaMalloc(&p, n * sizeof(T) + 16), "cudaMalloc");
    ptrs.push_back(p);
    return static_cast<T *>(p);
  }
  ~DeviceBuffers() {
    for (void *p : ptrs)
      cudaFree(p);
  }
};

} // namespace

void subpixel_rows(int dim, int cdir, int64_t npix, const double *lo, const double *hi, double tol, int maxeval,
                   int nobj, const mfd_object *objs, double eps_default, double *rows) {
  if (npix > (int64_t)0x7fffffff) throw Error("subpixel_rows: at most 2^31 - 1 pixels per call");
  const mgb_subpixel::SphereQuad &sq = mgb_subpixel::sphere_quadrature();
  DeviceBuffers b;
  double *dlo = b.alloc<double>(3 * npix), *dhi = b.alloc<double>(3 * npix), *drows = b.alloc<double>(3 * npix);
  double *dgrad = b.alloc<double>(3 * npix);
  int *dwork = b.alloc<int>(npix), *dnwork = b.alloc<int>(1);
  mfd_object *dobj = b.alloc<mfd_object>(nobj > 0 ? nobj : 1);
  mgb_subpixel::SphereQuad *dsq = b.alloc<mgb_subpixel::SphereQuad>(1);
  check(cudaMemcpy(dlo, lo, sizeof(double) * 3 * npix, cudaMemcpyHostToDevice), "copy pixels");
  check(cudaMemcpy(dhi, hi, sizeof(double) * 3 * npix, cudaMemcpyHostToDevice), "copy pixels");
  if (nobj > 0) check(cudaMemcpy(dobj, objs, sizeof(mfd_object) * nobj, cudaMemcpyHostToDevice), "copy objects");
  check(cudaMemcpy(dsq, &sq, sizeof(sq), cudaMemcpyHostToDevice), "copy quadrature");
  check(cudaMemset(dnwork, 0, sizeof(int)), "clear work count");
  const DeviceChi chi{dobj, nobj, eps_default};
  subpixel_normal_kernel<<<(unsigned)((npix + 127) / 128), 128>>>(dim, cdir, (long long)npix, dlo, dhi, maxeval,
                                                                   dsq, chi, drows, dgrad, dwork, dnwork);
  check(cudaGetLastError(), "subpixel_normal_kernel launch");
  int nwork = 0;
  check(cudaMemcpy(&nwork, dnwork, sizeof(int), cudaMemcpyDeviceToHost), "work count");
  if (nwork > 0) {
    int sms = 0, dev = 0;
    check(cudaGetDevice(&dev), "cudaGetDevice");
    check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
    // refinement levels: ms = 10, 20, 40, ... for the pixels still running
    LvState *dst = b.alloc<LvState>(npix);
    int *dnext = b.alloc<int>(nwork), *dover = b.alloc<int>(nwork), *dcount = b.alloc<int>(2);
    check(cudaMemset(dcount, 0, 2 * sizeof(int)), "clear counts");
    int *cur = dwork, *nxt = dnext, n = nwork, ms = 10, iter = 0, first = 1;
    while (n > 0) {
      const int ms2 = 2 * ms;
      iter += dim == 3 ? ms2 * ms2 * ms2 : ms2 * ms2;
      const int stop = maxeval && iter >= maxeval;
      check(cudaMemset(dcount, 0, sizeof(int)), "clear next count");
      const long long want = ((long long)n + 32 * LV_WARPS - 1) / (32 * LV_WARPS);
      const unsigned blocks = (unsigned)std::min<long long>(want, (long long)sms * 8);
      subpixel_level_kernel<<<blocks, 32 * LV_WARPS>>>(dim, cdir, dlo, dhi, tol, ms, first, stop, chi, dgrad, cur,
                                                       n, dst, nxt, dcount, dover, dcount + 1, drows);
      check(cudaGetLastError(), "subpixel_level_kernel launch");
      check(cudaMemcpy(&n, dcount, sizeof(int), cudaMemcpyDeviceToHost), "next count");
      std::swap(cur, nxt);
      ms = ms2;
      first = 0;
    }
    // pixels meeting too many objects: one warp each, all levels
    int nover = 0;
    check(cudaMemcpy(&nover, dcount + 1, sizeof(int), cudaMemcpyDeviceToHost), "overflow count");
    if (nover > 0) {
      const long long want = ((long long)nover + MEAN_WARPS - 1) / MEAN_WARPS;
      const unsigned blocks = (unsigned)std::min<long long>(want, (long long)sms * 16);
      subpixel_mean_kernel<<<blocks, 32 * MEAN_WARPS>>>(dim, cdir, dlo, dhi, tol, maxeval, chi, dgrad, dover,
                                                        dcount + 1, drows);
      check(cudaGetLastError(), "subpixel_mean_kernel launch");
    }
  }
  check(cudaMemcpy(rows, drows, sizeof(double) * 3 * npix, cudaMemcpyDeviceToHost), "copy rows");
}

} // namespace mfd
