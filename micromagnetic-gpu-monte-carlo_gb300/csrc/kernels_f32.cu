// kernels_f32.cu -- FP32 instantiation of the hot-path kernels (multiply-add
// contraction enabled).
#include "fused2d.cuh"
#include "grad.cuh"
#include "kernels.cuh"

namespace mmc {
MMC_INSTANTIATE_LAUNCHERS(float)
MMC_INSTANTIATE_FUSED(float)
MMC_INSTANTIATE_GRAD(float)
}  // namespace mmc
