// Fused-transform kernels for padded length(s) 24 48 (see fused_launch.cuh);
// one translation unit per size group so that they compile in parallel.
#include "fused_launch.cuh"

namespace mfx {
namespace ff {
MFX_FF_DEFINE(24)
MFX_FF_DEFINE(48)
}  // namespace ff
}  // namespace mfx
