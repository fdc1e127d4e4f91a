// Single-precision instantiation of the CUDA backend (FP32 fields and
// coefficients, FP64 DFT sums); fused multiply-adds allowed.
#include "mfd_cuda.cuh"

namespace mfd {

Backend *make_cuda_backend_f32(const Plan &p) { return new cuda_impl::CudaBackend<float>(p); }

} // namespace mfd
