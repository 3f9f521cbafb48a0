// The 3D moments pass on presampled images for f32 storage of the static
// ultrasound (patch radius 1-4), one translation unit per storage type.
#include "lc2_fused_ps.cuh"

namespace lc2 {
LC2_DEFINE_FUSED_PS(float)
}  // namespace lc2
