// rfgpu_mixed.cu - mixed-precision path (R = float): primitive state,
// gradients, limiter, reconstruction and flux arithmetic in FP32; residual
// sums compensated (TwoSum) in FP32, the conserved state a float-float pair
// updated without FP64 arithmetic, the record's EOS in FP32 with the energy's
// low part kept.  FP64 arithmetic only where a check or a transfer needs it
// (cells failing the positivity screen, the upload split, the download join
// and dv).  This unit is compiled with FMA contraction, the FP64 unit without.
#include "rfgpu_kernels.cuh"

namespace rfgpu {

RFGPU_INSTANTIATE(float)

}  // namespace rfgpu
