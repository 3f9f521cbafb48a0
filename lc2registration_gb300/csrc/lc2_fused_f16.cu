// Fused LC2 kernels for f16 storage (all patch radii), one translation unit
// per storage type so the instantiations compile in parallel.
#include "lc2_fused_ws.cuh"

namespace lc2 {
LC2_DEFINE_FUSED_LAUNCH(__half)
}  // namespace lc2
