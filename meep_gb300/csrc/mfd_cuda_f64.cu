// Double-precision instantiation of the CUDA backend.  Compiled with
// --fmad=false so every product and sum is rounded exactly as in the
// reference's default (non-FMA) x86-64 build; the FP64 path is the parity path.
#include "mfd_cuda.cuh"

namespace mfd {

Backend *make_cuda_backend_f32(const Plan &p);

Backend *make_backend(const Plan &p) {
  if (p.g.precision == 64) return new cuda_impl::CudaBackend<double>(p);
  return make_cuda_backend_f32(p);
}

} // namespace mfd
