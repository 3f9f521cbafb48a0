// Fused LC2 kernels of a resampled ultrasound (HighResolutionModality: Fixed)
// for f32 storage, one translation unit per storage type so the
// instantiations compile in parallel.
#include "lc2_fused_fixed.cuh"

namespace lc2 {
LC2_DEFINE_FIXED_LAUNCH(float)
}  // namespace lc2
