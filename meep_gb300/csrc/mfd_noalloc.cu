// Allocation-free flux reduction: the same sum as mfd_flux, F[w] =
// sum_k Re(E[k][w] conj(H[k][w])), with its scratch (per-block partial sums)
// in a file-scope device array instead of memory the engine allocates.
//
// Who needs it: callers that may not allocate device memory at the moment
// they reduce a spectrum -- hosts whose device memory is owned by another
// allocator (a framework's caching pool, a JVM/FFI host that hands out
// pre-allocated buffers), and latency-bound loops that cannot afford the
// implicit device synchronisation of cudaMalloc/cudaFree.  They pass device
// buffers in and out and a stream.
//
// Limits: nfreq <= MFD_NOALLOC_MAX_FREQ and the scratch holds at most
// MFD_NOALLOC_MAX_PARTS partial rows (larger monitors are folded into fewer,
// longer partial sums).  Every call on a device shares the one array, which
// keeps the last call's contents; each call overwrites every scratch entry it
// reads, so nothing needs clearing between calls.  Calls whose kernels
// overlap on the GPU (different streams without ordering) race on the scratch.
//
// Set-up: the first call on each device looks up the array's device address
// with cudaGetSymbolAddress (host code cannot use the symbol as a pointer), with
// that device current, and keeps it; make that first call before any stream
// capture.  The address is the device context's: after cudaDeviceReset the
// library has to be reloaded before it is called again.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <string>

#include "mfd.h"

namespace {

constexpr int kMaxFreq = MFD_NOALLOC_MAX_FREQ;
constexpr int kMaxParts = MFD_NOALLOC_MAX_PARTS;

// scratch: kMaxParts rows of kMaxFreq partial sums (2 MiB), resident on every
// device that loads this library until the process exits
static __device__ __align__(256) double g_flux_scratch[kMaxParts * kMaxFreq];

std::mutex g_mu;
double *g_scratch_ptr[64] = {};
thread_local std::string g_err;

__global__ void noalloc_partial_kernel(const double2 *E, const double2 *H, long long npts, int nf,
                                       double *partial) {
  const int w = blockIdx.x * 32 + threadIdx.x;
  double s = 0.0;
  if (w < nf)
    for (long long k = blockIdx.y * 8 + threadIdx.y; k < npts; k += 8LL * gridDim.y) {
      const double2 e = E[k * nf + w], h = H[k * nf + w];
      s += e.x * h.x + e.y * h.y;
    }
  __shared__ double red[8][33];
  red[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && w < nf) {
    double t = red[0][threadIdx.x];
    for (int r = 1; r < 8; r++)
      t += red[r][threadIdx.x];
    partial[(long long)blockIdx.y * nf + w] = t;
  }
}

__global__ void noalloc_final_kernel(const double *partial, int nparts, int nf, double *out) {
  const int w = blockIdx.x * 32 + threadIdx.x;
  double s = 0.0;
  if (w < nf)
    for (int q = threadIdx.y; q < nparts; q += 8)
      s += partial[(long long)q * nf + w];
  __shared__ double red[8][33];
  red[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && w < nf) {
    double t = red[0][threadIdx.x];
    for (int r = 1; r < 8; r++)
      t += red[r][threadIdx.x];
    out[w] = t;
  }
}

int fail(const std::string &m) {
  g_err = "meep: " + m;
  return -1;
}

} // namespace

extern "C" const char *mfd_noalloc_last_error(void) { return g_err.c_str(); }

extern "C" int mfd_flux_noalloc(const double *dft_E, const double *dft_H, int64_t npts, int nfreq,
                                double *flux_out, void *stream) {
  if (!dft_E || !dft_H || !flux_out) return fail("null device pointer");
  if (npts < 1 || nfreq < 1) return fail("npts and nfreq must be positive");
  if (nfreq > kMaxFreq)
    return fail("nfreq " + std::to_string(nfreq) + " exceeds the scratch limit of " +
                std::to_string(kMaxFreq) + " frequencies");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= 64) return fail("device ordinal out of range");
  double *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
      void *ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_flux_scratch);
      if (e != cudaSuccess) return fail(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_scratch_ptr[dev] = static_cast<double *>(ptr);
    }
    scratch = g_scratch_ptr[dev];
  }
  // partial rows: one per 1024 points, at most the scratch rows and what fits
  // kMaxParts * kMaxFreq for this nfreq
  long long rows = (npts + 1023) / 1024;
  long long cap = std::min<long long>(kMaxParts, (long long)kMaxParts * kMaxFreq / nfreq);
  int nparts = (int)std::max<long long>(1, std::min(rows, cap));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  dim3 grid((nfreq + 31) / 32, nparts), block(32, 8);
  noalloc_partial_kernel<<<grid, block, 0, st>>>(reinterpret_cast<const double2 *>(dft_E),
                                                 reinterpret_cast<const double2 *>(dft_H), npts, nfreq, scratch);
  noalloc_final_kernel<<<(nfreq + 31) / 32, block, 0, st>>>(scratch, nparts, nfreq, flux_out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(std::string("kernel launch: ") + cudaGetErrorString(e));
  return 0;
}
