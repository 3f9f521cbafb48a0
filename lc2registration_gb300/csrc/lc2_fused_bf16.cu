// Fused LC2 kernels for bf16 storage (all patch radii), one translation unit
// per storage type so the instantiations compile in parallel.
#include "lc2_fused_ws.cuh"

namespace lc2 {
LC2_DEFINE_FUSED_LAUNCH(__nv_bfloat16)
}  // namespace lc2
