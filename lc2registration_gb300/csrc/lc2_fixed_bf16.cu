// Fused LC2 kernels of a resampled ultrasound (HighResolutionModality: Fixed)
// for bf16 storage, one translation unit per storage type so the
// instantiations compile in parallel.
#include "lc2_fused_fixed.cuh"

namespace lc2 {
LC2_DEFINE_FIXED_LAUNCH(__nv_bfloat16)
}  // namespace lc2
