// Near-to-far transform on the GPU (mfd_near2far.cu): the far fields of the
// equivalent current sheets held by DFT monitors that already live in device
// memory.
#pragma once

#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "mfd_backend.hpp"

namespace mfd {

// one sheet with its device DFT sums (npts * nfreq complex, point-major)
struct N2FDevSheet {
  const double2 *dft;
  int n[3];          // points along x, y, z (1 for an absent direction)
  double is_half[3]; // see N2FSheet
  double rshift[3];
  int c0;
  long long start; // first flat source index of the sheet
  long long np;    // points
};

// out: nx * nf * 6 complex (re, im); freq: nf host frequencies.  Launches are
// counted into nlaunch; all work is ordered on `stream`.
void farfield_device(const N2FSpec &s, std::vector<N2FDevSheet> sheets, int nf, const double *freq, int64_t nx,
                     const double *x, double *out, cudaStream_t stream, long long &nlaunch);

// multiply n complex values in device memory by s
void scale_device(double2 *v, long long n, double sre, double sim, cudaStream_t stream, long long &nlaunch);

} // namespace mfd
