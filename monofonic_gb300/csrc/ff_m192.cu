// Fused-transform kernels for padded length(s) 192 (see fused_launch.cuh);
// one translation unit per size group so that they compile in parallel.
#include "fused_launch.cuh"

namespace mfx {
namespace ff {
MFX_FF_DEFINE(192)
}  // namespace ff
}  // namespace mfx
