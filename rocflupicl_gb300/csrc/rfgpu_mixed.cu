// rfgpu_mixed.cu - mixed-precision path: primitive state, gradients, limiter,
// reconstruction and flux arithmetic in FP32; residual accumulation, RK
// update, EOS and time step in FP64.
#include "rfgpu_kernels.cuh"

namespace rfgpu {

RFGPU_INSTANTIATE(float)

}  // namespace rfgpu
