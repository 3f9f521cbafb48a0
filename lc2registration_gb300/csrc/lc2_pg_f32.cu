// Fused 3D kernels on presampled images for f32 storage of the static
// ultrasound (patch radius 1-4), one translation unit per storage type.
#include "lc2_fused_pg.cuh"

namespace lc2 {
LC2_DEFINE_FUSED_PG(float)
}  // namespace lc2
