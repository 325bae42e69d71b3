// Fused-transform kernels for padded length(s) 96 (see fused_launch.cuh);
// one translation unit per size group so that they compile in parallel.
#include "fused_launch.cuh"

namespace mfx {
namespace ff {
MFX_FF_DEFINE(96)
}  // namespace ff
}  // namespace mfx
