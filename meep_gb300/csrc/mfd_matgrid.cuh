// Material grids on the device: the projected, interpolated design weights
// written into the diagonal chi1inv of the E components (one thread per Yee
// point of the block's index box), and the vector-Jacobian product dJ/du from
// dJ/dchi1inv over the design box.  The per-point arithmetic is matgrid.hpp,
// shared with the CPU oracle.
//
// The product is a gather: one thread per grid node visits the design points
// whose interpolation stencil can hold the node (a window of the box two
// nodes wide around it) in a fixed order, so the sums are reproducible; the
// per-point factor dJ/drho is formed first by a point kernel.
#pragma once

#include "matgrid.hpp"

namespace mfd {

struct MGPoints {
  int lo[3], n[3];   // index box of the component
  int io[3], sh[3];  // grid origin and the component's Yee shift (half pixels)
  int present[3];
  double inva;
  long long stride[3];
};

__device__ __forceinline__ void mg_point_x(const MGPoints &a, const int k[3], double x[3]) {
  for (int d = 0; d < 3; d++)
    x[d] = a.present[d] ? double(a.io[d] + a.sh[d] + 2 * k[d]) * (0.5 * a.inva) : 0.0;
}

__device__ __forceinline__ void mg_box_point(const MGPoints &a, long long t, int k[3]) {
  k[2] = a.lo[2] + int(t % a.n[2]);
  t /= a.n[2];
  k[1] = a.lo[1] + int(t % a.n[1]);
  k[0] = a.lo[0] + int(t / a.n[1]);
}

// the last of grids 0..ngrid-1 whose block holds x (-1 none)
__device__ __forceinline__ int mg_owner(const MatGridSpec *specs, int ngrid, const double x[3]) {
  for (int g = ngrid - 1; g >= 0; g--)
    if (mg_inside(specs[g], x)) return g;
  return -1;
}

template <typename R>
__global__ void matgrid_chi_kernel(MGPoints a, MatGridSpec s, const double *u, int d, R *chi) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)a.n[0] * a.n[1] * a.n[2]) return;
  int k[3];
  mg_box_point(a, t, k);
  double x[3], r[3];
  mg_point_x(a, k, x);
  if (!mg_inside(s, x)) return;
  mg_coords(s, x, r);
  const double up = mg_project(mg_interp(u, s.n, r), s.beta, s.eta);
  chi[k[0] * a.stride[0] + k[1] * a.stride[1] + k[2] * a.stride[2]] = R(1.0 / mg_eps(s, d, up));
}

// dJ/drho at every design point of one component (0 where grid id does not
// set the point)
static __global__ void matgrid_grho_kernel(MGPoints a, const MatGridSpec *specs, int ngrid, int id,
                                           const double *u, int d, const double *gchi, double *grho) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)a.n[0] * a.n[1] * a.n[2]) return;
  int k[3];
  mg_box_point(a, t, k);
  double x[3], r[3];
  mg_point_x(a, k, x);
  const double g = gchi[t];
  if (g == 0.0 || mg_owner(specs, ngrid, x) != id) {
    grho[t] = 0.0;
    return;
  }
  const MatGridSpec &s = specs[id];
  mg_coords(s, x, r);
  const double rho = mg_interp(u, s.n, r);
  const double eps = mg_eps(s, d, mg_project(rho, s.beta, s.eta));
  grho[t] = g * (-(s.eps2[d] - s.eps1[d]) / (eps * eps)) * mg_project_deriv(rho, s.beta, s.eta);
}

// weight of node i in the interpolation along one direction at block
// coordinate r (both stencil nodes may be i at a mirrored face)
__device__ __forceinline__ double mg_node_weight(double r, int n, int i) {
  int i1, i2;
  double w;
  mg_map(r, n, i1, i2, w);
  return (i1 == i ? 1.0 - w : 0.0) + (i2 == i ? w : 0.0);
}

// index window along d of the component's box points whose block coordinate
// lies in [(i - 1.5) / n, (i + 2.5) / n]: every point whose stencil can hold
// node i, with one index of margin
__device__ __forceinline__ void mg_window(const MGPoints &a, const MatGridSpec &s, int d, int i, int &k0,
                                          int &k1) {
  k0 = a.lo[d];
  k1 = a.lo[d] + a.n[d] - 1;
  if (!a.present[d] || s.size[d] == 0 || s.n[d] == 1) return;
  const double x0 = s.center[d] + ((i - 1.5) / s.n[d] - 0.5) * s.size[d];
  const double x1 = s.center[d] + ((i + 2.5) / s.n[d] - 0.5) * s.size[d];
  const double a2 = 2.0 / a.inva;
  const int w0 = int(floor((x0 * a2 - a.io[d] - a.sh[d]) / 2)) - 1;
  const int w1 = int(ceil((x1 * a2 - a.io[d] - a.sh[d]) / 2)) + 1;
  k0 = max(k0, w0);
  k1 = min(k1, w1);
}

// gu[node] (+)= sum over the component's points of grho * stencil weight
static __global__ void matgrid_gather_kernel(MGPoints a, MatGridSpec s, const double *grho, double *gu,
                                             int accumulate) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)s.n[0] * s.n[1] * s.n[2]) return;
  const int iz = int(t % s.n[2]), iy = int((t / s.n[2]) % s.n[1]), ix = int(t / ((long long)s.n[2] * s.n[1]));
  int lo[3], hi[3];
  mg_window(a, s, 0, ix, lo[0], hi[0]);
  mg_window(a, s, 1, iy, lo[1], hi[1]);
  mg_window(a, s, 2, iz, lo[2], hi[2]);
  double sum = 0.0;
  int k[3];
  for (k[0] = lo[0]; k[0] <= hi[0]; k[0]++)
    for (k[1] = lo[1]; k[1] <= hi[1]; k[1]++)
      for (k[2] = lo[2]; k[2] <= hi[2]; k[2]++) {
        const long long q = ((long long)(k[0] - a.lo[0]) * a.n[1] + (k[1] - a.lo[1])) * a.n[2] + (k[2] - a.lo[2]);
        const double g = grho[q];
        if (g == 0.0) continue;
        double x[3], r[3];
        mg_point_x(a, k, x);
        mg_coords(s, x, r);
        const double w = mg_node_weight(r[0], s.n[0], ix) * mg_node_weight(r[1], s.n[1], iy) *
                         mg_node_weight(r[2], s.n[2], iz);
        sum += g * w;
      }
  gu[t] = accumulate ? gu[t] + sum : sum;
}

} // namespace mfd
